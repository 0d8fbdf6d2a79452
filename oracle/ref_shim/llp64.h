/* Force-included (after msvc_compat.h) into BuildMatrix and Harm1D.
 *
 * Those programs were written for Windows (LLP64), where `long` is 4 bytes,
 * and they read and write the int32 binary mesh/SLAE files through `long*`.
 * On LP64 Linux that corrupts memory.  This header pulls in every system
 * header the programs use, then maps `long` to `int`, and routes the stdio
 * formatting calls through wrappers that rewrite the `%ld`-family
 * conversions to `%d` at run time, so the unmodified sources behave as they
 * do on Windows. */
#pragma once
#include <cstdio>
#include <cstdarg>
#include <cstdlib>
#include <cmath>
#include <ctime>
#include <omp.h>
#include <vector>
#include <iostream>
#include <fstream>
#include <sstream>
#include <algorithm>
#include <stack>
#include <complex>
#include <iomanip>
#include <string>
#include <stdexcept>
#include <iterator>
#include <set>
#include <map>

static inline const char *llp64_fix_format(const char *fmt, char *buf, size_t cap)
{
    size_t o = 0;
    for (size_t i = 0; fmt[i] != '\0' && o + 1 < cap; ++i) {
        buf[o++] = fmt[i];
        if (fmt[i] != '%') continue;
        /* copy flags / width / precision */
        size_t j = i + 1;
        while (fmt[j] != '\0' && strchr("-+ #0123456789.*", fmt[j]) && o + 1 < cap)
            buf[o++] = fmt[j++];
        if (fmt[j] == 'l' && fmt[j + 1] != '\0' && strchr("diuxXo", fmt[j + 1]))
            ++j; /* drop the 'l' length modifier: the argument is an int */
        i = j - 1;
    }
    buf[o] = '\0';
    return buf;
}
static inline int llp64_fscanf(FILE *f, const char *fmt, ...)
{
    char b[512]; va_list ap; va_start(ap, fmt);
    int r = vfscanf(f, llp64_fix_format(fmt, b, sizeof b), ap);
    va_end(ap); return r;
}
static inline int llp64_scanf(const char *fmt, ...)
{
    char b[512]; va_list ap; va_start(ap, fmt);
    int r = vscanf(llp64_fix_format(fmt, b, sizeof b), ap);
    va_end(ap); return r;
}
static inline int llp64_sscanf(const char *s, const char *fmt, ...)
{
    char b[512]; va_list ap; va_start(ap, fmt);
    int r = vsscanf(s, llp64_fix_format(fmt, b, sizeof b), ap);
    va_end(ap); return r;
}
static inline int llp64_fprintf(FILE *f, const char *fmt, ...)
{
    char b[512]; va_list ap; va_start(ap, fmt);
    int r = vfprintf(f, llp64_fix_format(fmt, b, sizeof b), ap);
    va_end(ap); return r;
}
static inline int llp64_printf(const char *fmt, ...)
{
    char b[512]; va_list ap; va_start(ap, fmt);
    int r = vprintf(llp64_fix_format(fmt, b, sizeof b), ap);
    va_end(ap); return r;
}
static inline int llp64_sprintf(char *s, const char *fmt, ...)
{
    char b[512]; va_list ap; va_start(ap, fmt);
    int r = vsprintf(s, llp64_fix_format(fmt, b, sizeof b), ap);
    va_end(ap); return r;
}
#define fscanf llp64_fscanf
#define scanf llp64_scanf
#define sscanf llp64_sscanf
#define fprintf llp64_fprintf
#define printf llp64_printf
#define sprintf llp64_sprintf
#define long int
