// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi)/2), a 48-bit significand computed entirely on
// the FP32 pipes.  GB300 issues FP32 at 64x its FP64 rate, so a few FP32
// operations per double-float operation still run far ahead of FP64.
//
// Error-free transformations used (Knuth's two-sum, Dekker's fast two-sum,
// the FMA two-product; see Shewchuk 1997, Hida-Li-Bailey 2001):
//   two_sum(a, b)      = (s, e) with s + e = a + b exactly      (6 flops)
//   fast_two_sum(a, b) = (s, e), requires |a| >= |b|            (3 flops)
//   two_prod(a, b)     = (p, e) with p + e = a * b exactly      (2 flops)
// Sums of products are accumulated unnormalised (hi carries a two-sum chain,
// lo collects the error terms) and normalised once at the end.
#pragma once
#include <cuda_runtime.h>

namespace mtgpu {
namespace dfl {

struct df {
    float h, l;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ df norm(float h, float l)
{
    df r;
    fast_two_sum(h, l, r.h, r.l);
    return r;
}

// unnormalised accumulator
struct acc {
    float h = 0.f, l = 0.f;
    __device__ __forceinline__ void add(df x)
    {
        float s, e;
        two_sum(h, x.h, s, e);
        h = s;
        l = __fadd_rn(l, __fadd_rn(e, x.l));
    }
    // += x * y
    __device__ __forceinline__ void mac(df x, df y)
    {
        const float p = __fmul_rn(x.h, y.h);
        float pe = __fmaf_rn(x.h, y.h, -p);
        pe = __fmaf_rn(x.h, y.l, pe);
        pe = __fmaf_rn(x.l, y.h, pe);
        float s, e;
        two_sum(h, p, s, e);
        h = s;
        l = __fadd_rn(l, __fadd_rn(e, pe));
    }
    // += x * y with y a plain float
    __device__ __forceinline__ void macf(df x, float y)
    {
        const float p = __fmul_rn(x.h, y);
        float pe = __fmaf_rn(x.h, y, -p);
        pe = __fmaf_rn(x.l, y, pe);
        float s, e;
        two_sum(h, p, s, e);
        h = s;
        l = __fadd_rn(l, __fadd_rn(e, pe));
    }
    __device__ __forceinline__ df get() const { return norm(h, l); }
    __device__ __forceinline__ double to_double() const { return (double)h + (double)l; }
};

__device__ __forceinline__ df neg(df a) { return df{-a.h, -a.l}; }

__device__ __forceinline__ df add(df a, df b)
{
    acc t;
    t.h = a.h;
    t.l = a.l;
    t.add(b);
    return t.get();
}

__device__ __forceinline__ df mul(df a, df b)
{
    acc t;
    t.mac(a, b);
    return t.get();
}

// complex double-float stored as float4 (re.h, re.l, im.h, im.l)
struct dfc {
    df re, im;
};

__device__ __forceinline__ dfc ld(const float4 *p, long long i)
{
    const float4 v = p[i];
    return dfc{df{v.x, v.y}, df{v.z, v.w}};
}
__device__ __forceinline__ void st(float4 *p, long long i, dfc v)
{
    p[i] = make_float4(v.re.h, v.re.l, v.im.h, v.im.l);
}

// x + a * y  (complex)
__device__ __forceinline__ dfc caxpy(dfc x, dfc a, dfc y)
{
    acc r, i;
    r.h = x.re.h; r.l = x.re.l;
    i.h = x.im.h; i.l = x.im.l;
    r.mac(a.re, y.re);
    r.mac(neg(a.im), y.im);
    i.mac(a.re, y.im);
    i.mac(a.im, y.re);
    return dfc{r.get(), i.get()};
}

__device__ __forceinline__ dfc cmul(dfc a, dfc b)
{
    acc r, i;
    r.mac(a.re, b.re);
    r.mac(neg(a.im), b.im);
    i.mac(a.re, b.im);
    i.mac(a.im, b.re);
    return dfc{r.get(), i.get()};
}

// host/device conversion of an FP64 value (host side or rare device use)
__host__ __device__ __forceinline__ df from_double(double v)
{
    const float h = (float)v;
    return df{h, (float)(v - (double)h)};
}

}  // namespace dfl
}  // namespace mtgpu
