// dfloat.h -- double-float ("float-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// i.e. a ~48-bit significand.  The operations are the error-free
// transformations of Knuth (TwoSum), Dekker (Fast2Sum) and the fused
// multiply-add product (TwoProd = a*b and fma(a, b, -a*b)), combined as in
// Dekker (1971) and in the double-double literature (Hida, Li and Bailey,
// "Library for double-double and quad-double arithmetic", 2001), here with
// float halves.  Additions are the "sloppy" form (one TwoSum of the high
// parts): their error is ~2^-47 of the larger operand.
//
// The translation unit that includes this header must be compiled without
// FMA contraction (nvcc --fmad=false): the error-free transformations rely
// on every product and sum being rounded where the source says, and every
// fused multiply-add here is an explicit fmaf().  The header also compiles as
// plain C++ (no CUDA), so its accuracy can be checked on the host.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

// DFO: kept out of line on the device.  The integrator's loop is far larger than
// an SM's instruction cache, and one shared copy of these longer operations (in
// place of one per call site) took 3.6 % off its time; results are the same.
#ifdef __CUDACC__
#define DFI __host__ __device__ __forceinline__
#define DFO inline __host__ __device__ __noinline__
#else
#define DFI inline
#define DFO inline
#endif

namespace etraj {

struct df {
    float hi, lo;
};

DFI df df_f(float h) { return df{h, 0.0f}; }

// s + e = a + b exactly (Knuth's TwoSum)
DFI df two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return df{s, (a - (s - bb)) + (b - bb)};
}
// s + e = a + b exactly, given |a| >= |b| or a == 0 (Dekker's Fast2Sum)
DFI df quick_two_sum(float a, float b) {
    const float s = a + b;
    return df{s, b - (s - a)};
}
// p + e = a * b exactly
DFI df two_prod(float a, float b) {
    const float p = a * b;
    return df{p, fmaf(a, b, -p)};
}

// nearest double-float of an FP64 value (FP64 operations: use at load/store only)
DFI df df_from_double(double x) {
    const float h = (float)x;
    return df{h, (float)(x - (double)h)};
}
DFI double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

DFI df df_neg(df a) { return df{-a.hi, -a.lo}; }
DFI df df_abs(df a) { return a.hi < 0.0f ? df{-a.hi, -a.lo} : a; }

DFI df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return quick_two_sum(s.hi, s.lo);
}
DFI df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
DFI df df_add_f(df a, float b) {
    df s = two_sum(a.hi, b);
    s.lo += a.lo;
    return quick_two_sum(s.hi, s.lo);
}
DFI df df_mul(df a, df b) {
    df p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return quick_two_sum(p.hi, p.lo);
}
DFI df df_mul_f(df a, float b) {
    df p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return quick_two_sum(p.hi, p.lo);
}
DFI df df_sqr(df a) {
    df p = two_prod(a.hi, a.hi);
    p.lo = fmaf(a.hi + a.hi, a.lo, p.lo);
    return quick_two_sum(p.hi, p.lo);
}
// a * b + c with one renormalization
DFI df df_fma(df a, df b, df c) {
    df p = two_prod(a.hi, b.hi);
    const float e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    df s = two_sum(p.hi, c.hi);
    s.lo += e + c.lo;
    return quick_two_sum(s.hi, s.lo);
}
// a * b + c for a float a
DFI df df_fma_f(float a, df b, df c) {
    df p = two_prod(a, b.hi);
    const float e = fmaf(a, b.lo, p.lo);
    df s = two_sum(p.hi, c.hi);
    s.lo += e + c.lo;
    return quick_two_sum(s.hi, s.lo);
}
DFO df df_div(df a, df b) {
    const float q1 = a.hi / b.hi;
    // r = a - q1 b; a.hi - q1 b.hi is exact (the two are within a factor of 2)
    df p = two_prod(q1, b.hi);
    p.lo = fmaf(q1, b.lo, p.lo);
    const float r = ((a.hi - p.hi) - p.lo) + a.lo;
    return quick_two_sum(q1, r / b.hi);
}
DFO df df_rcp(df b) {
    const float q1 = 1.0f / b.hi;
    df p = two_prod(q1, b.hi);
    p.lo = fmaf(q1, b.lo, p.lo);
    const float r = (1.0f - p.hi) - p.lo;
    return quick_two_sum(q1, r * q1);
}
DFO df df_sqrt(df a) {
    if (!(a.hi > 0.0f)) return df{0.0f, 0.0f};
    const float s = sqrtf(a.hi);
    const df p = two_prod(s, s);
    const float r = ((a.hi - p.hi) - p.lo) + a.lo;
    return quick_two_sum(s, r * (0.5f / s));
}
// 1 / sqrt(a), a > 0
DFI df df_rsqrt(df a) { return df_rcp(df_sqrt(a)); }

DFI bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
DFI df df_min(df a, df b) { return df_lt(b, a) ? b : a; }
DFI df df_max(df a, df b) { return df_lt(a, b) ? b : a; }

// ---- exp, exp2, log2 -------------------------------------------------------------------
// Tang's table method (ACM TOMS 15, 1989) in double-float: x = (256 m + j) ln2/256 + r
// with |r| <= ln2/512, exp(x) = 2^m 2^(j/256) exp(r).  For exp, ln2/256 is split in
// three floats (Cody-Waite) so that n ln2/256 is exact to ~2^-60 for |n| < 2^15.
// The 256 table entries 2^(j/256) are double-float values (ETRAJ_DF_EXP2_TABLE).
constexpr float kExpInvL = 0x1.715476p+8f;      // 256 / ln 2
constexpr float kExpL1 = 0x1.63p-9f;             // ln2/256, first 9 bits
constexpr float kExpL2 = -0x1.bd0106p-21f;       // next 24 bits
constexpr float kExpL3 = 0x1.cf78p-48f;          // the rest
constexpr int kExpTabN = 256;
constexpr int kLogTabN = 128;
constexpr df kDfLn2 = {0x1.62e43p-1f, -0x1.05c61p-29f};
constexpr df kDfInvLn2 = {0x1.715476p+0f, 0x1.4ae0cp-26f};
constexpr df kDfLog2Of10 = {0x1.a934fp+1f, 0x1.2f346ep-24f};

// 2^(j/256), j = 0..255, as double-float (hi, lo) pairs: hi is the float nearest the
// value (computed to 60 digits), lo the float nearest the remainder.
#define ETRAJ_DF_EXP2_TABLE \
    0x1.0000000000000p+0f, 0.0f, 0x1.00b1b00000000p+0f, -0x1.6950d00000000p-26f, \
    0x1.0163da0000000p+0f, 0x1.3f66660000000p-25f, 0x1.0216820000000p+0f, -0x1.789fb00000000p-25f, \
    0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f, 0x1.037d420000000p+0f, 0x1.c2377a0000000p-25f, \
    0x1.04315e0000000p+0f, 0x1.0dcff00000000p-25f, 0x1.04e5f80000000p+0f, -0x1.a1356a0000000p-25f, \
    0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f, 0x1.0650a00000000p+0f, 0x1.c783f20000000p-25f, \
    0x1.0706b20000000p+0f, 0x1.3bbedc0000000p-25f, 0x1.07bd420000000p+0f, 0x1.6e55060000000p-25f, \
    0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f, 0x1.092be00000000p+0f, -0x1.333f040000000p-25f, \
    0x1.09e3ec0000000p+0f, 0x1.58de700000000p-25f, 0x1.0a9c7a0000000p+0f, -0x1.3831ba0000000p-26f, \
    0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f, 0x1.0c0f140000000p+0f, 0x1.791b220000000p-26f, \
    0x1.0cc9220000000p+0f, 0x1.6e48fe0000000p-25f, 0x1.0d83b20000000p+0f, 0x1.9caef60000000p-27f, \
    0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f, 0x1.0efa560000000p+0f, -0x1.02b1da0000000p-31f, \
    0x1.0fb66a0000000p+0f, 0x1.ffda640000000p-25f, 0x1.1073020000000p+0f, 0x1.1ae4680000000p-25f, \
    0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f, 0x1.11edba0000000p+0f, 0x1.6bc5560000000p-25f, \
    0x1.12abdc0000000p+0f, 0x1.b0c7300000000p-30f, 0x1.136a820000000p+0f, -0x1.61bf6a0000000p-25f, \
    0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f, 0x1.14e95a0000000p+0f, -0x1.9619da0000000p-25f, \
    0x1.15a98c0000000p+0f, 0x1.14b1ca0000000p-25f, 0x1.166a460000000p+0f, -0x1.71c7880000000p-25f, \
    0x1.172b840000000p+0f, -0x1.c157420000000p-27f, 0x1.17ed480000000p+0f, 0x1.a56ef00000000p-26f, \
    0x1.18af940000000p+0f, -0x1.dcdc860000000p-26f, 0x1.1972660000000p+0f, -0x1.f228b40000000p-26f, \
    0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f, 0x1.1af9a00000000p+0f, -0x1.fb1d780000000p-26f, \
    0x1.1bbe080000000p+0f, 0x1.0117340000000p-26f, 0x1.1c82fa0000000p+0f, -0x1.5afc720000000p-25f, \
    0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f, 0x1.1e0e760000000p+0f, -0x1.4bbfda0000000p-28f, \
    0x1.1ed5020000000p+0f, 0x1.7e6c8e0000000p-27f, 0x1.1f9c180000000p+0f, 0x1.0e33940000000p-26f, \
    0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f, 0x1.212be40000000p+0f, -0x1.50eafc0000000p-25f, \
    0x1.21f49a0000000p+0f, -0x1.d0446e0000000p-25f, 0x1.22bdda0000000p+0f, 0x1.3c89680000000p-27f, \
    0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f, 0x1.2452000000000p+0f, -0x1.1f7afe0000000p-26f, \
    0x1.251ce40000000p+0f, 0x1.f654c80000000p-25f, 0x1.25e8580000000p+0f, -0x1.dc26320000000p-25f, \
    0x1.26b4560000000p+0f, 0x1.789f380000000p-26f, 0x1.2780e40000000p+0f, -0x1.7c441a0000000p-25f, \
    0x1.284dfe0000000p+0f, 0x1.f563800000000p-28f, 0x1.291ba80000000p+0f, -0x1.4dc8920000000p-25f, \
    0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f, 0x1.2ab8a60000000p+0f, 0x1.b443c40000000p-26f, \
    0x1.2b87fe0000000p+0f, -0x1.e4a4ce0000000p-25f, 0x1.2c57e40000000p+0f, -0x1.a239340000000p-26f, \
    0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f, 0x1.2df9620000000p+0f, -0x1.37d4ee0000000p-29f, \
    0x1.2ecafa0000000p+0f, 0x1.27c5ea0000000p-25f, 0x1.2f9d240000000p+0f, 0x1.57b10e0000000p-25f, \
    0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f, 0x1.31432e0000000p+0f, 0x1.bdd6600000000p-25f, \
    0x1.3217100000000p+0f, -0x1.d993e80000000p-27f, 0x1.32eb840000000p+0f, -0x1.15c5740000000p-26f, \
    0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f, 0x1.3496260000000p+0f, 0x1.b8fe8c0000000p-26f, \
    0x1.356c560000000p+0f, -0x1.b5803c0000000p-30f, 0x1.36431a0000000p+0f, 0x1.6f441e0000000p-27f, \
    0x1.371a740000000p+0f, -0x1.18aac60000000p-25f, 0x1.37f2620000000p+0f, 0x1.8f3aa40000000p-27f, \
    0x1.38cae60000000p+0f, 0x1.a0bb0c0000000p-25f, 0x1.39a4020000000p+0f, -0x1.23afc40000000p-26f, \
    0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f, 0x1.3b57fc0000000p+0f, -0x1.3930ba0000000p-32f, \
    0x1.3c32dc0000000p+0f, 0x1.89d4720000000p-27f, 0x1.3d0e540000000p+0f, 0x1.3b785c0000000p-26f, \
    0x1.3dea640000000p+0f, 0x1.8246840000000p-25f, 0x1.3ec70e0000000p+0f, -0x1.c75d160000000p-29f, \
    0x1.3fa4500000000p+0f, 0x1.2b20060000000p-26f, 0x1.40822c0000000p+0f, 0x1.b3d0120000000p-27f, \
    0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f, 0x1.423fb20000000p+0f, 0x1.c251a20000000p-26f, \
    0x1.431f5e0000000p+0f, -0x1.abd5da0000000p-26f, 0x1.43ffa40000000p+0f, -0x1.ed18b00000000p-30f, \
    0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f, 0x1.45c2040000000p+0f, 0x1.53e9180000000p-27f, \
    0x1.46a41e0000000p+0f, 0x1.a3a00a0000000p-25f, 0x1.4786d60000000p+0f, 0x1.a2cc8e0000000p-26f, \
    0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f, 0x1.494e1e0000000p+0f, 0x1.92aed20000000p-28f, \
    0x1.4a32b00000000p+0f, -0x1.e505840000000p-25f, 0x1.4b17de0000000p+0f, 0x1.4db6fa0000000p-25f, \
    0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f, 0x1.4ce41c0000000p+0f, -0x1.fa0fba0000000p-26f, \
    0x1.4dcb2a0000000p+0f, -0x1.8088bc0000000p-26f, 0x1.4eb2d80000000p+0f, 0x1.d8abfe0000000p-28f, \
    0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f, 0x1.5084180000000p+0f, -0x1.759c240000000p-29f, \
    0x1.516daa0000000p+0f, 0x1.67b3200000000p-27f, 0x1.5257de0000000p+0f, 0x1.07e9de0000000p-25f, \
    0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f, 0x1.542e300000000p+0f, -0x1.612a5c0000000p-25f, \
    0x1.551a4c0000000p+0f, 0x1.4bb2420000000p-25f, 0x1.56070e0000000p+0f, -0x1.0b77980000000p-27f, \
    0x1.56f4740000000p+0f, -0x1.295b040000000p-25f, 0x1.57e27e0000000p+0f, -0x1.074ecc0000000p-26f, \
    0x1.58d12e0000000p+0f, -0x1.6d07000000000p-25f, 0x1.59c0820000000p+0f, 0x1.ffc1f20000000p-26f, \
    0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f, 0x1.5ba1200000000p+0f, -0x1.15e1800000000p-26f, \
    0x1.5c92680000000p+0f, 0x1.4b28d60000000p-25f, 0x1.5d845a0000000p+0f, -0x1.ecce8e0000000p-25f, \
    0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f, 0x1.5f6a320000000p+0f, 0x1.b9d6e20000000p-29f, \
    0x1.605e1c0000000p+0f, -0x1.a248fe0000000p-26f, 0x1.6152ae0000000p+0f, 0x1.b37dbe0000000p-26f, \
    0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f, 0x1.633dd20000000p+0f, -0x1.736b020000000p-27f, \
    0x1.6434640000000p+0f, -0x1.66679c0000000p-25f, 0x1.652ba00000000p+0f, -0x1.43704a0000000p-28f, \
    0x1.6623880000000p+0f, 0x1.2a91120000000p-27f, 0x1.671c1c0000000p+0f, 0x1.c20cfe0000000p-26f, \
    0x1.68155e0000000p+0f, -0x1.766ad20000000p-25f, 0x1.690f4c0000000p+0f, -0x1.cc2d580000000p-25f, \
    0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f, 0x1.6b05300000000p+0f, -0x1.62ba300000000p-26f, \
    0x1.6c01280000000p+0f, -0x1.5e84a80000000p-25f, 0x1.6cfdce0000000p+0f, -0x1.15c4de0000000p-27f, \
    0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f, 0x1.6ef92a0000000p+0f, -0x1.e9b1460000000p-26f, \
    0x1.6ff7e00000000p+0f, -0x1.ab9ae00000000p-26f, 0x1.70f7460000000p+0f, 0x1.bd0ba20000000p-26f, \
    0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f, 0x1.72f8280000000p+0f, 0x1.bab4220000000p-26f, \
    0x1.73f9a40000000p+0f, 0x1.14b02e0000000p-25f, 0x1.74fbd40000000p+0f, -0x1.4506800000000p-25f, \
    0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f, 0x1.77024c0000000p+0f, -0x1.ca923e0000000p-25f, \
    0x1.7806940000000p+0f, 0x1.fbcba80000000p-25f, 0x1.790b940000000p+0f, -0x1.d4f8c20000000p-26f, \
    0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f, 0x1.7b17b00000000p+0f, 0x1.2ed9fc0000000p-25f, \
    0x1.7c1ed00000000p+0f, 0x1.30c1320000000p-28f, 0x1.7d26a60000000p+0f, 0x1.7fc3780000000p-27f, \
    0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f, 0x1.7f38780000000p+0f, 0x1.2471240000000p-26f, \
    0x1.8042760000000p+0f, -0x1.783cbe0000000p-25f, 0x1.814d2a0000000p+0f, 0x1.ba20dc0000000p-25f, \
    0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f, 0x1.8364c20000000p+0f, -0x1.46be080000000p-28f, \
    0x1.8471a40000000p+0f, 0x1.88f1ec0000000p-26f, 0x1.857f420000000p+0f, -0x1.0c149c0000000p-25f, \
    0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f, 0x1.879cae0000000p+0f, -0x1.b396f20000000p-26f, \
    0x1.88ac7e0000000p+0f, -0x1.9d665a0000000p-26f, 0x1.89bd0a0000000p+0f, 0x1.1e16040000000p-26f, \
    0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f, 0x1.8be05c0000000p+0f, -0x1.4a7a220000000p-26f, \
    0x1.8cf3220000000p+0f, -0x1.29576e0000000p-25f, 0x1.8e06a60000000p+0f, -0x1.f799280000000p-28f, \
    0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f, 0x1.902fee0000000p+0f, -0x1.fafa6e0000000p-25f, \
    0x1.9145b00000000p+0f, 0x1.723ff80000000p-25f, 0x1.925c360000000p+0f, -0x1.8aba040000000p-25f, \
    0x1.93737c0000000p+0f, -0x1.e647440000000p-25f, 0x1.948b820000000p+0f, 0x1.6bf31c0000000p-25f, \
    0x1.95a44c0000000p+0f, 0x1.790a420000000p-25f, 0x1.96bdda0000000p+0f, -0x1.6263d40000000p-26f, \
    0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f, 0x1.98f33e0000000p+0f, 0x1.1e88a80000000p-26f, \
    0x1.9a0f180000000p+0f, -0x1.e6bf080000000p-25f, 0x1.9b2bb40000000p+0f, 0x1.aa7fc20000000p-25f, \
    0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f, 0x1.9d67420000000p+0f, -0x1.ad11ca0000000p-26f, \
    0x1.9e86320000000p+0f, -0x1.8737380000000p-26f, 0x1.9fa5e80000000p+0f, 0x1.a0fe540000000p-25f, \
    0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f, 0x1.a1e7ae0000000p+0f, 0x1.b1d7180000000p-25f, \
    0x1.a309be0000000p+0f, 0x1.8945a60000000p-25f, 0x1.a42c980000000p+0f, 0x1.182b5e0000000p-30f, \
    0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f, 0x1.a674a80000000p+0f, 0x1.5e8c0a0000000p-25f, \
    0x1.a799e20000000p+0f, -0x1.99e9940000000p-25f, 0x1.a8bfe60000000p+0f, -0x1.87da340000000p-25f, \
    0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f, 0x1.ab0e520000000p+0f, 0x1.356eba0000000p-28f, \
    0x1.ac36bc0000000p+0f, -0x1.6064320000000p-31f, 0x1.ad5ff40000000p+0f, -0x1.70f6220000000p-26f, \
    0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f, 0x1.afb4ce0000000p+0f, 0x1.88bcc00000000p-26f, \
    0x1.b0e0720000000p+0f, 0x1.31b6cc0000000p-25f, 0x1.b20ce60000000p+0f, 0x1.93512a0000000p-25f, \
    0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f, 0x1.b468420000000p+0f, -0x1.4916ca0000000p-25f, \
    0x1.b597280000000p+0f, 0x1.bcab280000000p-25f, 0x1.b6c6e20000000p+0f, 0x1.3e38a60000000p-25f, \
    0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f, 0x1.b928d00000000p+0f, -0x1.bb16c40000000p-25f, \
    0x1.ba5b040000000p+0f, -0x1.ebdf360000000p-25f, 0x1.bb8e0c0000000p+0f, -0x1.0cb21c0000000p-25f, \
    0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f, 0x1.bdf69c0000000p+0f, 0x1.f9d1040000000p-27f, \
    0x1.bf2c260000000p+0f, -0x1.0a387e0000000p-26f, 0x1.c062860000000p+0f, 0x1.41b33c0000000p-28f, \
    0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f, 0x1.c2d1ce0000000p+0f, -0x1.8166b60000000p-26f, \
    0x1.c40ab60000000p+0f, -0x1.7c2c980000000p-39f, 0x1.c544780000000p+0f, -0x1.c141380000000p-26f, \
    0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f, 0x1.c7ba880000000p+0f, 0x1.3119260000000p-25f, \
    0x1.c8f6da0000000p+0f, -0x1.7f230a0000000p-25f, 0x1.ca34060000000p+0f, -0x1.15c7640000000p-25f, \
    0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f, 0x1.ccb0f20000000p+0f, 0x1.cda2ce0000000p-25f, \
    0x1.cdf0b60000000p+0f, -0x1.5447800000000p-25f, 0x1.cf31560000000p+0f, -0x1.2915240000000p-26f, \
    0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f, 0x1.d1b5320000000p+0f, 0x1.61192e0000000p-25f, \
    0x1.d2f8700000000p+0f, 0x1.01b13e0000000p-25f, 0x1.d43c8e0000000p+0f, 0x1.59543a0000000p-25f, \
    0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f, 0x1.d6c76e0000000p+0f, 0x1.0c5cda0000000p-25f, \
    0x1.d80e320000000p+0f, -0x1.26cf8e0000000p-25f, 0x1.d955d80000000p+0f, -0x1.c013f20000000p-25f, \
    0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f, 0x1.dbe7ce0000000p+0f, -0x1.38af9e0000000p-25f, \
    0x1.dd32200000000p+0f, -0x1.9fc9740000000p-25f, 0x1.de7d560000000p+0f, 0x1.0701960000000p-26f, \
    0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f, 0x1.e116760000000p+0f, 0x1.632fa20000000p-25f, \
    0x1.e264620000000p+0f, -0x1.614bda0000000p-25f, 0x1.e3b3340000000p+0f, -0x1.3a447c0000000p-26f, \
    0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f, 0x1.e653920000000p+0f, 0x1.19db5e0000000p-26f, \
    0x1.e7a5200000000p+0f, -0x1.0e2ce00000000p-26f, 0x1.e8f7980000000p+0f, -0x1.0649180000000p-25f, \
    0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f, 0x1.eb9f480000000p+0f, 0x1.9f329c0000000p-26f, \
    0x1.ecf4820000000p+0f, 0x1.b1ccfe0000000p-25f, 0x1.ee4aaa0000000p+0f, 0x1.0c42880000000p-27f, \
    0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f, 0x1.f0f9c20000000p+0f, -0x1.a4df6c0000000p-27f, \
    0x1.f252b40000000p+0f, -0x1.1288ae0000000p-25f, 0x1.f3ac940000000p+0f, 0x1.1bae4e0000000p-25f, \
    0x1.f507660000000p+0f, -0x1.246eb00000000p-26f, 0x1.f663280000000p+0f, -0x1.9deec20000000p-26f, \
    0x1.f7bfda0000000p+0f, 0x1.b397c20000000p-25f, 0x1.f91d800000000p+0f, 0x1.121e440000000p-27f, \
    0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f, 0x1.fbdba40000000p+0f, -0x1.2da55e0000000p-25f, \
    0x1.fd3c220000000p+0f, 0x1.71ee3e0000000p-25f, 0x1.fe9d960000000p+0f, 0x1.65447c0000000p-25f
// log2(c_j), c_j = 1 + (j + 1/2)/128, j = 0..127, as double-float pairs (60 digits, rounded)
#define ETRAJ_DF_LOG2C_TABLE \
    0x1.709c460000000p-8f, 0x1.af558e0000000p-33f, 0x1.1363120000000p-6f, -0x1.0ad09e0000000p-31f, \
    0x1.c9363c0000000p-6f, -0x1.5ebc1e0000000p-32f, 0x1.3ed30a0000000p-5f, -0x1.72f4bc0000000p-30f, \
    0x1.985bfc0000000p-5f, 0x1.a4a8ca0000000p-32f, 0x1.f138980000000p-5f, 0x1.9929d00000000p-32f, \
    0x1.24b5b80000000p-4f, -0x1.eca5c40000000p-32f, 0x1.507b840000000p-4f, -0x1.3f988a0000000p-29f, \
    0x1.7beeea0000000p-4f, -0x1.28ebb00000000p-29f, 0x1.a7111e0000000p-4f, -0x1.96f6d80000000p-33f, \
    0x1.d1e34e0000000p-4f, 0x1.adc16e0000000p-31f, 0x1.fc66a00000000p-4f, 0x1.e160140000000p-29f, \
    0x1.134e1c0000000p-3f, -0x1.6edf3a0000000p-28f, 0x1.2842940000000p-3f, 0x1.60f4c80000000p-28f, \
    0x1.3d11460000000p-3f, 0x1.b3514c0000000p-28f, 0x1.51baba0000000p-3f, -0x1.f0b46e0000000p-28f, \
    0x1.663f700000000p-3f, -0x1.4dbb3a0000000p-29f, 0x1.7a9fec0000000p-3f, 0x1.f417780000000p-29f, \
    0x1.8edcae0000000p-3f, 0x1.06a56e0000000p-28f, 0x1.a2f6320000000p-3f, 0x1.905c360000000p-30f, \
    0x1.b6ecf20000000p-3f, -0x1.140d420000000p-28f, 0x1.cac1640000000p-3f, -0x1.c4791c0000000p-30f, \
    0x1.de73fe0000000p-3f, 0x1.d8a4080000000p-30f, 0x1.f205340000000p-3f, -0x1.b7dc360000000p-29f, \
    0x1.02baba0000000p-2f, 0x1.2683320000000p-29f, 0x1.0c62980000000p-2f, -0x1.557aae0000000p-27f, \
    0x1.15fa680000000p-2f, -0x1.289ee00000000p-27f, 0x1.1f82600000000p-2f, -0x1.24ee3e0000000p-27f, \
    0x1.28fab40000000p-2f, -0x1.499b300000000p-27f, 0x1.3263960000000p-2f, 0x1.b5941a0000000p-29f, \
    0x1.3bbd3a0000000p-2f, 0x1.43b9f60000000p-31f, 0x1.4507d00000000p-2f, -0x1.22b03c0000000p-30f, \
    0x1.4e43880000000p-2f, 0x1.d1f6d40000000p-31f, 0x1.5770920000000p-2f, -0x1.3321ce0000000p-28f, \
    0x1.608f1c0000000p-2f, -0x1.7ad6ea0000000p-27f, 0x1.699f520000000p-2f, 0x1.23352e0000000p-28f, \
    0x1.72a1640000000p-2f, -0x1.0687d00000000p-27f, 0x1.7b957a0000000p-2f, 0x1.8a35580000000p-27f, \
    0x1.847bc40000000p-2f, -0x1.84f3ce0000000p-27f, 0x1.8d54680000000p-2f, -0x1.8947920000000p-27f, \
    0x1.961f900000000p-2f, 0x1.49d0260000000p-28f, 0x1.9edd680000000p-2f, -0x1.4c9b440000000p-27f, \
    0x1.a78e140000000p-2f, 0x1.bdefbe0000000p-28f, 0x1.b031be0000000p-2f, 0x1.fc0c860000000p-27f, \
    0x1.b8c88e0000000p-2f, -0x1.01de620000000p-28f, 0x1.c152a60000000p-2f, 0x1.84995c0000000p-27f, \
    0x1.c9d0300000000p-2f, -0x1.26b70a0000000p-27f, 0x1.d2414c0000000p-2f, 0x1.017e500000000p-27f, \
    0x1.daa6220000000p-2f, 0x1.0327dc0000000p-29f, 0x1.e2fed40000000p-2f, -0x1.7b46b40000000p-29f, \
    0x1.eb4b840000000p-2f, 0x1.f456f40000000p-28f, 0x1.f38c560000000p-2f, 0x1.ef31500000000p-28f, \
    0x1.fbc16c0000000p-2f, -0x1.bf65fe0000000p-28f, 0x1.01f5720000000p-1f, 0x1.dc99380000000p-27f, \
    0x1.0604720000000p-1f, -0x1.836c540000000p-27f, 0x1.0a0dc40000000p-1f, -0x1.60e3c00000000p-26f, \
    0x1.0e11780000000p-1f, -0x1.56507e0000000p-26f, 0x1.120f9e0000000p-1f, -0x1.8c3d000000000p-26f, \
    0x1.1608440000000p-1f, 0x1.2578020000000p-27f, 0x1.19fb7c0000000p-1f, -0x1.c336f80000000p-27f, \
    0x1.1de9520000000p-1f, -0x1.31a22c0000000p-28f, 0x1.21d1d60000000p-1f, -0x1.124a9a0000000p-27f, \
    0x1.25b5160000000p-1f, -0x1.d230be0000000p-27f, 0x1.2993200000000p-1f, -0x1.30dd540000000p-26f, \
    0x1.2d6c020000000p-1f, -0x1.95fd900000000p-26f, 0x1.313fc80000000p-1f, 0x1.4366de0000000p-26f, \
    0x1.350e840000000p-1f, -0x1.b51f040000000p-26f, 0x1.38d83e0000000p-1f, 0x1.7ae84a0000000p-32f, \
    0x1.3c9d060000000p-1f, 0x1.242b840000000p-27f, 0x1.405ce80000000p-1f, 0x1.a71e980000000p-26f, \
    0x1.4417f20000000p-1f, 0x1.32085a0000000p-27f, 0x1.47ce300000000p-1f, -0x1.a5fb500000000p-26f, \
    0x1.4b7fac0000000p-1f, -0x1.06da1a0000000p-27f, 0x1.4f2c740000000p-1f, 0x1.a9f33e0000000p-29f, \
    0x1.52d4940000000p-1f, 0x1.723c840000000p-28f, 0x1.5678180000000p-1f, -0x1.1e53f40000000p-27f, \
    0x1.5a170a0000000p-1f, 0x1.2fe3580000000p-27f, 0x1.5db1780000000p-1f, -0x1.5ef7d80000000p-26f, \
    0x1.61476a0000000p-1f, 0x1.8d88440000000p-32f, 0x1.64d8ee0000000p-1f, -0x1.11cc820000000p-26f, \
    0x1.68660c0000000p-1f, 0x1.2dedf00000000p-26f, 0x1.6beed20000000p-1f, 0x1.2866d80000000p-28f, \
    0x1.6f73480000000p-1f, 0x1.78b8c20000000p-26f, 0x1.72f37a0000000p-1f, 0x1.a298b60000000p-26f, \
    0x1.766f720000000p-1f, 0x1.64c7be0000000p-26f, 0x1.79e73a0000000p-1f, 0x1.1200c40000000p-26f, \
    0x1.7d5adc0000000p-1f, 0x1.681e2a0000000p-27f, 0x1.80ca620000000p-1f, 0x1.a537e40000000p-31f, \
    0x1.8435d60000000p-1f, -0x1.66b9120000000p-26f, 0x1.879d400000000p-1f, -0x1.c262480000000p-28f, \
    0x1.8b00aa0000000p-1f, 0x1.e2da960000000p-26f, 0x1.8e60200000000p-1f, 0x1.11eb300000000p-28f, \
    0x1.91bba80000000p-1f, 0x1.23e2e20000000p-26f, 0x1.95134e0000000p-1f, -0x1.4f63a40000000p-26f, \
    0x1.9867180000000p-1f, -0x1.24b8fa0000000p-26f, 0x1.9bb7100000000p-1f, -0x1.528c6c0000000p-27f, \
    0x1.9f033e0000000p-1f, 0x1.991d2a0000000p-26f, 0x1.a24bae0000000p-1f, -0x1.2300920000000p-26f, \
    0x1.a590640000000p-1f, 0x1.1315640000000p-29f, 0x1.a8d16c0000000p-1f, -0x1.d03b180000000p-26f, \
    0x1.ac0eca0000000p-1f, 0x1.9322680000000p-26f, 0x1.af488c0000000p-1f, -0x1.5d0da60000000p-26f, \
    0x1.b27eb40000000p-1f, 0x1.7f1e120000000p-26f, 0x1.b5b1500000000p-1f, -0x1.ee0d340000000p-26f, \
    0x1.b8e0620000000p-1f, 0x1.10e6120000000p-30f, 0x1.bc0bf60000000p-1f, -0x1.01b9400000000p-26f, \
    0x1.bf34120000000p-1f, -0x1.d7736c0000000p-26f, 0x1.c258bc0000000p-1f, 0x1.59920a0000000p-27f, \
    0x1.c579fe0000000p-1f, 0x1.76b6ca0000000p-26f, 0x1.c897e00000000p-1f, -0x1.7c929c0000000p-27f, \
    0x1.cbb2660000000p-1f, 0x1.333f3e0000000p-27f, 0x1.cec99a0000000p-1f, -0x1.23adfe0000000p-29f, \
    0x1.d1dd820000000p-1f, -0x1.92cf040000000p-27f, 0x1.d4ee240000000p-1f, 0x1.59718a0000000p-27f, \
    0x1.d7fb8a0000000p-1f, -0x1.ec9ab20000000p-26f, 0x1.db05b60000000p-1f, 0x1.145f6c0000000p-26f, \
    0x1.de0cb40000000p-1f, -0x1.a331d60000000p-27f, 0x1.e110860000000p-1f, 0x1.b5ee920000000p-26f, \
    0x1.e411360000000p-1f, 0x1.d5caa80000000p-26f, 0x1.e70eca0000000p-1f, 0x1.1fbe1c0000000p-27f, \
    0x1.ea09480000000p-1f, -0x1.4238780000000p-26f, 0x1.ed00b40000000p-1f, 0x1.117d840000000p-26f, \
    0x1.eff5180000000p-1f, 0x1.5fa7c80000000p-30f, 0x1.f2e6780000000p-1f, 0x1.7eb8460000000p-29f, \
    0x1.f5d4da0000000p-1f, 0x1.9de6d80000000p-26f, 0x1.f8c0460000000p-1f, 0x1.e746340000000p-28f, \
    0x1.fba8c00000000p-1f, 0x1.7151380000000p-27f, 0x1.fe8e500000000p-1f, -0x1.d485cc0000000p-26f
// 1/c_j of the same points, as double-float pairs
#define ETRAJ_DF_RCPC_TABLE \
    0x1.fe01fe0000000p-1f, 0x1.fe01fe0000000p-33f, 0x1.fa11ca0000000p-1f, 0x1.403f420000000p-26f, \
    0x1.f6310a0000000p-1f, 0x1.941b760000000p-26f, 0x1.f25f640000000p-1f, 0x1.08c2ae0000000p-27f, \
    0x1.ee9c800000000p-1f, -0x1.ee9c800000000p-27f, 0x1.eae8080000000p-1f, -0x1.517f860000000p-27f, \
    0x1.e741aa0000000p-1f, 0x1.65d43a0000000p-27f, 0x1.e3a9180000000p-1f, -0x1.88f9640000000p-27f, \
    0x1.e01e020000000p-1f, -0x1.fe1fe20000000p-29f, 0x1.dca01e0000000p-1f, -0x1.aff11a0000000p-28f, \
    0x1.d92f220000000p-1f, 0x1.8f3fc40000000p-28f, 0x1.d5cac80000000p-1f, 0x1.d5cac80000000p-31f, \
    0x1.d272ca0000000p-1f, 0x1.fe2d8e0000000p-28f, 0x1.cf26e60000000p-1f, -0x1.dda01c0000000p-28f, \
    0x1.cbe6da0000000p-1f, -0x1.3fc6840000000p-26f, 0x1.c8b2660000000p-1f, -0x1.411d700000000p-27f, \
    0x1.c5894e0000000p-1f, -0x1.de56d00000000p-26f, 0x1.c26b540000000p-1f, -0x1.b457f80000000p-27f, \
    0x1.bf583e0000000p-1f, 0x1.d0d1b20000000p-26f, 0x1.bc4fd60000000p-1f, 0x1.620f9e0000000p-27f, \
    0x1.b951e20000000p-1f, 0x1.631fe40000000p-26f, 0x1.b65e2e0000000p-1f, 0x1.df77020000000p-28f, \
    0x1.b374840000000p-1f, 0x1.5b00da0000000p-26f, 0x1.b094b40000000p-1f, -0x1.c4dbac0000000p-26f, \
    0x1.adbe880000000p-1f, -0x1.adbe880000000p-31f, 0x1.aaf1d20000000p-1f, 0x1.f0fd800000000p-26f, \
    0x1.a82e660000000p-1f, -0x1.d9e3d40000000p-26f, 0x1.a574100000000p-1f, 0x1.da22920000000p-27f, \
    0x1.a2c2a80000000p-1f, 0x1.f147280000000p-27f, 0x1.a01a020000000p-1f, -0x1.7f97fa0000000p-27f, \
    0x1.9d79f20000000p-1f, -0x1.1292fa0000000p-26f, 0x1.9ae24e0000000p-1f, 0x1.4aa21c0000000p-26f, \
    0x1.9852f00000000p-1f, 0x1.b1d8200000000p-26f, 0x1.95cbb00000000p-1f, 0x1.7c6ef60000000p-26f, \
    0x1.934c680000000p-1f, -0x1.934c680000000p-31f, 0x1.90d4f20000000p-1f, -0x1.bfcde60000000p-26f, \
    0x1.8e65280000000p-1f, -0x1.43b2300000000p-27f, 0x1.8bfce80000000p-1f, 0x1.8bfce80000000p-31f, \
    0x1.899c100000000p-1f, -0x1.3fcecc0000000p-26f, 0x1.87427c0000000p-1f, -0x1.9fb6a40000000p-28f, \
    0x1.84f00c0000000p-1f, 0x1.3c030a0000000p-28f, 0x1.82a4a00000000p-1f, 0x1.82a4a00000000p-29f, \
    0x1.8060180000000p-1f, 0x1.8060180000000p-31f, 0x1.7e22560000000p-1f, -0x1.d4b61c0000000p-26f, \
    0x1.7beb3a0000000p-1f, -0x1.ba3fd00000000p-26f, 0x1.79baa60000000p-1f, 0x1.76c7320000000p-26f, \
    0x1.7790820000000p-1f, -0x1.cca73e0000000p-26f, 0x1.756cac0000000p-1f, 0x1.00bab60000000p-28f, \
    0x1.734f0c0000000p-1f, 0x1.507fa40000000p-27f, 0x1.7137860000000p-1f, 0x1.b38f820000000p-26f, \
    0x1.6f26020000000p-1f, -0x1.21b3fe0000000p-26f, 0x1.6d1a620000000p-1f, 0x1.a072180000000p-27f, \
    0x1.6b14900000000p-1f, 0x1.5463480000000p-26f, 0x1.6914740000000p-1f, -0x1.5dcbd00000000p-27f, \
    0x1.6719f40000000p-1f, -0x1.3fd31c0000000p-26f, 0x1.6524f80000000p-1f, 0x1.4ed2a80000000p-27f, \
    0x1.63356c0000000p-1f, -0x1.dd4fc80000000p-27f, 0x1.614b360000000p-1f, 0x1.0635d20000000p-26f, \
    0x1.5f66440000000p-1f, -0x1.7ada400000000p-26f, 0x1.5d867c0000000p-1f, 0x1.f671520000000p-28f, \
    0x1.5babcc0000000p-1f, 0x1.91fea40000000p-27f, 0x1.59d6200000000p-1f, -0x1.db866a0000000p-26f, \
    0x1.5805600000000p-1f, 0x1.5805600000000p-29f, 0x1.56397c0000000p-1f, -0x1.60eb480000000p-27f, \
    0x1.54725e0000000p-1f, 0x1.aee0c00000000p-27f, 0x1.52aff60000000p-1f, -0x1.2aff560000000p-26f, \
    0x1.50f22e0000000p-1f, 0x1.11c4c60000000p-29f, 0x1.4f38f60000000p-1f, 0x1.6ea64e0000000p-28f, \
    0x1.4d843c0000000p-1f, -0x1.23d3b40000000p-29f, 0x1.4bd3ee0000000p-1f, -0x1.2cb8100000000p-28f, \
    0x1.4a27fa0000000p-1f, 0x1.aec02a0000000p-26f, 0x1.4880520000000p-1f, 0x1.00a4400000000p-28f, \
    0x1.46dce40000000p-1f, -0x1.74d3f40000000p-26f, 0x1.453d9e0000000p-1f, 0x1.63bb660000000p-28f, \
    0x1.43a2740000000p-1f, -0x1.ea82360000000p-26f, 0x1.420b520000000p-1f, 0x1.9796540000000p-27f, \
    0x1.40782e0000000p-1f, -0x1.de33540000000p-26f, 0x1.3ee8f40000000p-1f, 0x1.52d7840000000p-28f, \
    0x1.3d5d9a0000000p-1f, -0x1.cab1480000000p-26f, 0x1.3bd60e0000000p-1f, -0x1.b735aa0000000p-27f, \
    0x1.3a52440000000p-1f, -0x1.e14df80000000p-27f, 0x1.38d22e0000000p-1f, -0x1.933eee0000000p-26f, \
    0x1.3755be0000000p-1f, -0x1.c6d7420000000p-26f, 0x1.35dce60000000p-1f, -0x1.8354200000000p-31f, \
    0x1.34679a0000000p-1f, 0x1.9c02680000000p-26f, 0x1.32f5ce0000000p-1f, 0x1.ad43c00000000p-26f, \
    0x1.3187760000000p-1f, -0x1.c585120000000p-27f, 0x1.301c820000000p-1f, 0x1.58804c0000000p-26f, \
    0x1.2eb4ea0000000p-1f, 0x1.fed14c0000000p-29f, 0x1.2d50a00000000p-1f, 0x1.2d50a00000000p-29f, \
    0x1.2bef980000000p-1f, 0x1.cb46e20000000p-26f, 0x1.2a91ca0000000p-1f, -0x1.a187e00000000p-26f, \
    0x1.2937260000000p-1f, -0x1.11fed60000000p-27f, 0x1.27dfa40000000p-1f, -0x1.d78c6c0000000p-27f, \
    0x1.268b380000000p-1f, -0x1.94ff6c0000000p-28f, 0x1.2539d80000000p-1f, -0x1.6e884e0000000p-29f, \
    0x1.23eb7a0000000p-1f, -0x1.1d13f40000000p-26f, 0x1.22a0120000000p-1f, 0x1.5009160000000p-28f, \
    0x1.2157980000000p-1f, 0x1.2157980000000p-31f, 0x1.2012020000000p-1f, -0x1.bfdbfe0000000p-26f, \
    0x1.1ecf440000000p-1f, -0x1.c023da0000000p-28f, 0x1.1d8f560000000p-1f, 0x1.cb92b00000000p-27f, \
    0x1.1c52300000000p-1f, -0x1.f18fd40000000p-28f, 0x1.1b17c60000000p-1f, 0x1.fcaeb80000000p-27f, \
    0x1.19e0120000000p-1f, -0x1.87fb980000000p-27f, 0x1.18ab080000000p-1f, 0x1.c815ee0000000p-28f, \
    0x1.1778a20000000p-1f, -0x1.b90a5e0000000p-27f, 0x1.1648d60000000p-1f, -0x1.e079c00000000p-26f, \
    0x1.151b9a0000000p-1f, 0x1.feeae40000000p-28f, 0x1.13f0e80000000p-1f, 0x1.a688e40000000p-26f, \
    0x1.12c8b80000000p-1f, 0x1.3db8160000000p-26f, 0x1.11a3020000000p-1f, -0x1.962df60000000p-27f, \
    0x1.107fbc0000000p-1f, -0x1.feef800000000p-29f, 0x1.0f5ee00000000p-1f, -0x1.5336980000000p-27f, \
    0x1.0e40660000000p-1f, -0x1.4fb3fe0000000p-26f, 0x1.0d24460000000p-1f, -0x1.394c380000000p-26f, \
    0x1.0c0a780000000p-1f, 0x1.a2d05c0000000p-27f, 0x1.0af2f80000000p-1f, -0x1.ba226a0000000p-26f, \
    0x1.09ddba0000000p-1f, 0x1.abe0d80000000p-27f, 0x1.08cabc0000000p-1f, -0x1.9153440000000p-26f, \
    0x1.07b9f20000000p-1f, 0x1.371d5c0000000p-26f, 0x1.06ab5a0000000p-1f, -0x1.c376820000000p-28f, \
    0x1.059eea0000000p-1f, 0x1.c9d61a0000000p-31f, 0x1.04949c0000000p-1f, 0x1.82cc980000000p-26f, \
    0x1.038c6c0000000p-1f, -0x1.0fb7000000000p-26f, 0x1.0286500000000p-1f, -0x1.c46b0c0000000p-28f, \
    0x1.0182440000000p-1f, -0x1.35d0ba0000000p-26f, 0x1.0080400000000p-1f, 0x1.0080400000000p-28f

constexpr float kExp2Tab[2 * kExpTabN] = {ETRAJ_DF_EXP2_TABLE};
constexpr float kLog2cTab[2 * kLogTabN] = {ETRAJ_DF_LOG2C_TABLE};
constexpr float kRcpcTab[2 * kLogTabN] = {ETRAJ_DF_RCPC_TABLE};

// exp(r) - 1 for |r| <= ~1.4e-3: r + r^2/2 in double-float, r^3/6 + r^4/24 in FP32
// (below 4.2e-10 and 1.4e-13), the truncation r^5/120 < 4e-17
DFI df df_expm1_small(df r) {
    df r2 = df_sqr(r);
    r2.hi *= 0.5f;
    r2.lo *= 0.5f;
    const float tail = (r.hi * r.hi) * (r.hi * fmaf(r.hi, 1.0f / 24.0f, 1.0f / 6.0f));
    return df_add_f(df_add(r, r2), tail);
}
// 2^(j/256) (1 + p) 2^m for -126 <= m <= 127, n = 256 m + j
DFI df df_exp_assemble(int n, df p, const float* tab) {
    const int j = n & (kExpTabN - 1);
    const int m = n >> 8;  // floor(n / 256)
    const df T = df{tab[2 * j], tab[2 * j + 1]};
    const df e = df_fma(T, p, T);
    const uint32_t bits = (uint32_t)(m + 127) << 23;
    float sc;
    std::memcpy(&sc, &bits, sizeof sc);
    return df{e.hi * sc, e.lo * sc};
}

// exp(x) for x <= 0 (results below 2^-126 are returned as 0); tab: ETRAJ_DF_EXP2_TABLE
DFI df df_exp_neg(df x, const float* tab) {
    if (!(x.hi > -87.0f)) return df{0.0f, 0.0f};
    const float n = rintf(x.hi * kExpInvL);
    // r = x - n ln2/256: x.hi - n L1 is exact (n L1 has <= 24 bits and is within a
    // factor of 2 of x.hi, or r is tiny)
    df r = two_sum(fmaf(-n, kExpL1, x.hi), x.lo);
    r = df_add(r, two_prod(-n, kExpL2));
    r.lo = fmaf(-n, kExpL3, r.lo);
    r = quick_two_sum(r.hi, r.lo);
    return df_exp_assemble((int)n, df_expm1_small(r), tab);
}

// 2^x for -126 <= x < 127: x = n/256 + r (x.hi - n/256 is exact), |r| <= 1/512,
// 2^r = exp(r ln 2); outside the range the result is clamped to 0 or 2^127.
DFO df df_exp2(df x, const float* tab) {
    if (!(x.hi >= -126.0f)) return df{0.0f, 0.0f};
    if (x.hi >= 127.0f) return df{0x1p127f, 0.0f};
    const float n = rintf(x.hi * 256.0f);
    const df r = two_sum(fmaf(-n, 0.00390625f, x.hi), x.lo);
    return df_exp_assemble((int)n, df_expm1_small(df_mul(r, kDfLn2)), tab);
}

// log2(x) for a normal x > 0: x = 2^e m with m in [1, 2), m = c_j (1 + r) with c_j the
// centre of m's 1/128 subinterval (m.hi - c_j is exact), |r| <= 1/256, and
// log(1 + r) = r - r^2/2 (double-float) + r^3/3 - r^4/4 + r^5/5 - r^6/6 (FP32, below
// 2e-8; truncation r^7/7 < 2e-18).  log2c, rcpc: ETRAJ_DF_LOG2C_TABLE, ETRAJ_DF_RCPC_TABLE.
DFO df df_log2(df x, const float* log2c, const float* rcpc) {
    uint32_t bits;
    std::memcpy(&bits, &x.hi, sizeof bits);
    const int e = (int)((bits >> 23) & 0xffu) - 127;
    const int j = (int)((bits >> 16) & 0x7fu);
    const uint32_t mbits = (bits & 0x007fffffu) | 0x3f800000u;
    float mh;
    std::memcpy(&mh, &mbits, sizeof mh);
    const uint32_t sbits = (uint32_t)(127 - e) << 23;  // 2^-e, -126 <= e <= 127
    float sc;
    std::memcpy(&sc, &sbits, sizeof sc);
    const float c = 1.0f + ((float)j + 0.5f) * 0.0078125f;
    const df d = two_sum(mh - c, x.lo * sc);
    const df r = df_mul(d, df{rcpc[2 * j], rcpc[2 * j + 1]});
    df r2 = df_sqr(r);
    r2.hi *= -0.5f;
    r2.lo *= -0.5f;
    const float a = r.hi;
    const float tail = (a * a) * (a * fmaf(a, fmaf(a, fmaf(a, -1.0f / 6.0f, 0.2f), -0.25f), 1.0f / 3.0f));
    const df l = df_add_f(df_add(r, r2), tail);
    return df_add(df_add_f(df{log2c[2 * j], log2c[2 * j + 1]}, (float)e), df_mul(l, kDfInvLn2));
}

}  // namespace etraj
