// gw_math64.cuh -- FP64 exp and log for the global step's lane program.
//
// On GB300 a warp's FP64 instruction occupies its SM sub-partition's FP64 unit for ~64 cycles, with
// or without instruction-level parallelism, so the global step costs about 64 cycles per FP64
// instruction of its busiest warp.  These two functions use table-driven reductions with few FP64
// operations (11 for exp, 13 for log):
//   exp: Tang, "Table-driven implementation of the exponential function in IEEE floating-point
//        arithmetic", ACM TOMS 15(2), 1989 -- x = (64 m + j) ln2/64 + r, |r| <= ln2/128,
//        exp(x) = 2^m 2^(j/64) (1 + p(r)), p the degree-5 Taylor polynomial of exp(r) - 1.
//   log: Tang, "Table-driven implementation of the logarithm function in IEEE floating-point
//        arithmetic", ACM TOMS 16(4), 1990 -- x = 2^e m, F = 1 + (j + 1/2)/128 from the leading
//        7 fraction bits, u = m invF - 1 (one FMA), log(x) = e ln2 - log(invF) + log1p(u), log1p
//        by its degree-7 Taylor polynomial (|u| < 2^-8).
// Inputs outside the reduced ranges (|x| >= 700 for exp; non-positive, non-normal, non-finite
// or within 2^-5 of 1 for log) take CUDA's exp / log.  Domain tests use integer compares on the
// bit patterns, so they cost no FP64 issue slots.  Tables (generated by gen_math_tables.py from
// 60-digit decimal arithmetic) are copied to shared memory once per launch.
#pragma once

#include <cuda_runtime.h>

#include "gw_math_tables.h"

namespace gw {
namespace math64 {

struct Tables {
    double e2[64][2];   // 2^(j/64) lead, trail
    double lg[128][3];  // invF_j, -log(invF_j) lead, trail
};

static __constant__ double c_exp2_table[64][2] = GW_EXP2_TABLE;
static __constant__ double c_log_table[128][3] = GW_LOG_TABLE;

// Copies the tables to shared memory; threads tid = 0 .. n-1 of the caller take part.
__device__ __forceinline__ void load_tables(Tables &T, int tid, int n) {
    for (int i = tid; i < 64 * 2; i += n) (&T.e2[0][0])[i] = (&c_exp2_table[0][0])[i];
    for (int i = tid; i < 128 * 3; i += n) (&T.lg[0][0])[i] = (&c_log_table[0][0])[i];
}

__device__ __forceinline__ double exp(double x, const Tables &T) {
    const unsigned long long ax = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
    if (ax >= 0x4085E00000000000ull) return ::exp(x);  // |x| >= 700, inf, NaN
    const double shifter = 0x1.8p52;
    const double t = fma(x, k64ByLn2, shifter);  // k = round(64 x / ln2) in the low bits of t
    const double kd = t - shifter;
    const int k = __double2loint(t);
    double r = fma(-kd, kLn2By64Hi, x);
    r = fma(-kd, kLn2By64Lo, r);
    double a = fma(r, 1.0 / 120.0, 1.0 / 24.0);
    a = fma(r, a, 1.0 / 6.0);
    a = fma(r, a, 0.5);
    const double r2 = r * r;
    const double p = fma(r2, a, r);  // exp(r) - 1
    const int j = k & 63, m = k >> 6;
    const double sl = T.e2[j][0], st = T.e2[j][1];
    const double res = sl + fma(sl, p, st);
    // res * 2^m (|m| <= 1010: the result stays normal)
    return __hiloint2double(__double2hiint(res) + (m << 20), __double2loint(res));
}

__device__ __forceinline__ double log(double x, const Tables &T) {
    const long long b = __double_as_longlong(x);
    // positive normal finite and not within 2^-5 of 1 (there log(x) is small and the reduction
    // would cancel)
    const bool normal = (unsigned long long)(b - 0x0010000000000000ll) < 0x7FE0000000000000ull;
    const bool near1 = (unsigned long long)(b - 0x3FEF000000000000ll) < 0x0001800000000000ull;
    if (!normal || near1) return ::log(x);
    const int hi = (int)(b >> 32);
    const int e = ((hi >> 20) & 0x7FF) - 1023;
    const int j = (hi >> 13) & 0x7F;
    const double m = __longlong_as_double((b & 0x000FFFFFFFFFFFFFll) | 0x3FF0000000000000ll);
    const double u = fma(m, T.lg[j][0], -1.0);
    double a = fma(u, 1.0 / 7.0, -1.0 / 6.0);
    a = fma(u, a, 0.2);
    a = fma(u, a, -0.25);
    a = fma(u, a, 1.0 / 3.0);
    a = fma(u, a, -0.5);
    const double q = fma(u * u, a, u);  // log1p(u)
    const double ed = (double)e;
    const double h = fma(ed, kLn2Hi, T.lg[j][1]);
    const double l = fma(ed, kLn2Lo, T.lg[j][2]) + q;
    return h + l;
}

}  // namespace math64
}  // namespace gw
