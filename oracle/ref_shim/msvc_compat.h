/* Force-included into every reference translation unit built by
 * oracle/build_ref.sh.  It supplies the few MSVC-only names the reference
 * uses so that g++ on Linux can compile the sources where they lie,
 * unmodified. */
#pragma once
#include <cstring>
#include <cstdio>
#include <ctime>
#include <cerrno>
#define __forceinline inline
typedef long long __time64_t;
static inline __time64_t _time64(__time64_t *t)
{
    __time64_t v = (__time64_t)time(nullptr);
    if (t) *t = v;
    return v;
}
static inline int memcpy_s(void *dst, size_t dst_size, const void *src, size_t n)
{
    if (n > dst_size) return ERANGE;
    memcpy(dst, src, n);
    return 0;
}
