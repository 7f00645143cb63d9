/*
 * immintrin.h -- a portable stand-in for the x86 SIMD intrinsics header, for
 * compiling the reference's numerical core on hosts without AVX (the aarch64
 * GPU hosts).  TEST INFRASTRUCTURE ONLY: it is put first on the include path
 * of the checker build (oracle/Makefile, target ref on a non-x86 host), so
 * the reference's own `#include <immintrin.h>` resolves here and its sources
 * compile unmodified.
 *
 * Each intrinsic is written from its documented semantics (Intel Intrinsics
 * Guide) on GCC vector extensions: 256-bit vectors of four doubles, 128-bit
 * vectors of two.  Only the intrinsics the reference uses are provided.  The
 * fused multiply-adds are one rounding (std::fma), as AVX2's FMA3 is; max
 * returns its second operand unless the first is larger (NaN and equal
 * operands give the second), as MAXPD does; compares give all-ones lanes.
 */
#ifndef FCS_SIMD_SHIM_IMMINTRIN_H
#define FCS_SIMD_SHIM_IMMINTRIN_H

#include <math.h>
#include <stdint.h>
#include <string.h>

typedef double __m256d __attribute__((vector_size(32), __may_alias__));
typedef long long __m256i __attribute__((vector_size(32), __may_alias__));
typedef double __m128d __attribute__((vector_size(16), __may_alias__));
typedef long long __shim_m128i __attribute__((vector_size(16), __may_alias__));

#define _CMP_LT_OQ 0x11
#define _CMP_GE_OQ 0x1d
#define _MM_SHUFFLE(z, y, x, w) (((z) << 6) | ((y) << 4) | ((x) << 2) | (w))

#define SHIM_INLINE static inline __attribute__((always_inline))

/* ---- 256-bit: construction, loads, stores ---- */
SHIM_INLINE __m256d _mm256_set1_pd(double a) { __m256d r = {a, a, a, a}; return r; }
SHIM_INLINE __m256d _mm256_setr_pd(double a, double b, double c, double d) { __m256d r = {a, b, c, d}; return r; }
SHIM_INLINE __m256d _mm256_setzero_pd(void) { __m256d r = {0.0, 0.0, 0.0, 0.0}; return r; }
SHIM_INLINE __m256i _mm256_set1_epi64x(long long a) { __m256i r = {a, a, a, a}; return r; }
SHIM_INLINE __m256d _mm256_loadu_pd(const double* p) { __m256d r; memcpy(&r, p, sizeof r); return r; }
SHIM_INLINE void _mm256_storeu_pd(double* p, __m256d a) { memcpy(p, &a, sizeof a); }
SHIM_INLINE __m256d _mm256_castsi256_pd(__m256i a) { return (__m256d)a; }
SHIM_INLINE __m128d _mm256_castpd256_pd128(__m256d a) { __m128d r = {a[0], a[1]}; return r; }
SHIM_INLINE __m128d _mm256_extractf128_pd(__m256d a, const int imm) {
    __m128d r = {a[(imm & 1) * 2], a[(imm & 1) * 2 + 1]};
    return r;
}
SHIM_INLINE double _mm256_cvtsd_f64(__m256d a) { return a[0]; }

/* ---- 256-bit arithmetic ---- */
SHIM_INLINE __m256d _mm256_add_pd(__m256d a, __m256d b) { return a + b; }
SHIM_INLINE __m256d _mm256_sub_pd(__m256d a, __m256d b) { return a - b; }
SHIM_INLINE __m256d _mm256_mul_pd(__m256d a, __m256d b) { return a * b; }
SHIM_INLINE __m256d _mm256_div_pd(__m256d a, __m256d b) { return a / b; }
SHIM_INLINE __m256d _mm256_fmadd_pd(__m256d a, __m256d b, __m256d c) {
    __m256d r = {fma(a[0], b[0], c[0]), fma(a[1], b[1], c[1]), fma(a[2], b[2], c[2]), fma(a[3], b[3], c[3])};
    return r;
}
SHIM_INLINE __m256d _mm256_fmsub_pd(__m256d a, __m256d b, __m256d c) {
    __m256d r = {fma(a[0], b[0], -c[0]), fma(a[1], b[1], -c[1]), fma(a[2], b[2], -c[2]), fma(a[3], b[3], -c[3])};
    return r;
}
SHIM_INLINE __m256d _mm256_max_pd(__m256d a, __m256d b) {
    __m256d r;
    for (int i = 0; i < 4; i++) r[i] = a[i] > b[i] ? a[i] : b[i];
    return r;
}
SHIM_INLINE __m256d _mm256_hadd_pd(__m256d a, __m256d b) {
    __m256d r = {a[0] + a[1], b[0] + b[1], a[2] + a[3], b[2] + b[3]};
    return r;
}

/* ---- 256-bit compares, selects, bit operations, permutes ---- */
SHIM_INLINE __m256d _mm256_cmp_pd(__m256d a, __m256d b, const int pred) {
    __m256i m;
    for (int i = 0; i < 4; i++) {
        const int t = pred == _CMP_LT_OQ ? (a[i] < b[i]) : pred == _CMP_GE_OQ ? (a[i] >= b[i]) : 0;
        m[i] = t ? -1LL : 0LL;
    }
    return (__m256d)m;
}
SHIM_INLINE __m256d _mm256_blendv_pd(__m256d a, __m256d b, __m256d mask) {
    const __m256i m = (__m256i)mask;
    __m256d r;
    for (int i = 0; i < 4; i++) r[i] = m[i] < 0 ? b[i] : a[i];
    return r;
}
SHIM_INLINE __m256d _mm256_andnot_pd(__m256d a, __m256d b) { return (__m256d)(~(__m256i)a & (__m256i)b); }
SHIM_INLINE __m256d _mm256_permute4x64_pd(__m256d a, const int imm) {
    __m256d r = {a[imm & 3], a[(imm >> 2) & 3], a[(imm >> 4) & 3], a[(imm >> 6) & 3]};
    return r;
}
SHIM_INLINE __m256d _mm256_permute2f128_pd(__m256d a, __m256d b, const int imm) {
    __m256d r;
    for (int h = 0; h < 2; h++) {
        const int c = (imm >> (4 * h)) & 0xf;
        const __m256d src = (c & 2) ? b : a;
        const int off = (c & 1) * 2;
        r[2 * h] = (c & 8) ? 0.0 : src[off];
        r[2 * h + 1] = (c & 8) ? 0.0 : src[off + 1];
    }
    return r;
}

/* ---- 128-bit ---- */
SHIM_INLINE __m128d _mm_set1_pd(double a) { __m128d r = {a, a}; return r; }
SHIM_INLINE __m128d _mm_setr_pd(double a, double b) { __m128d r = {a, b}; return r; }
SHIM_INLINE __m128d _mm_setzero_pd(void) { __m128d r = {0.0, 0.0}; return r; }
SHIM_INLINE __m128d _mm_loadu_pd(const double* p) { __m128d r; memcpy(&r, p, sizeof r); return r; }
SHIM_INLINE void _mm_storeu_pd(double* p, __m128d a) { memcpy(p, &a, sizeof a); }
SHIM_INLINE void _mm_store_sd(double* p, __m128d a) { *p = a[0]; }
SHIM_INLINE double _mm_cvtsd_f64(__m128d a) { return a[0]; }
SHIM_INLINE __m128d _mm_add_pd(__m128d a, __m128d b) { return a + b; }
SHIM_INLINE __m128d _mm_mul_pd(__m128d a, __m128d b) { return a * b; }
SHIM_INLINE __m128d _mm_div_pd(__m128d a, __m128d b) { return a / b; }
SHIM_INLINE __m128d _mm_add_sd(__m128d a, __m128d b) { __m128d r = {a[0] + b[0], a[1]}; return r; }
SHIM_INLINE __m128d _mm_fmadd_pd(__m128d a, __m128d b, __m128d c) {
    __m128d r = {fma(a[0], b[0], c[0]), fma(a[1], b[1], c[1])};
    return r;
}
SHIM_INLINE __m128d _mm_max_pd(__m128d a, __m128d b) {
    __m128d r = {a[0] > b[0] ? a[0] : b[0], a[1] > b[1] ? a[1] : b[1]};
    return r;
}
SHIM_INLINE __m128d _mm_max_sd(__m128d a, __m128d b) { __m128d r = {a[0] > b[0] ? a[0] : b[0], a[1]}; return r; }
SHIM_INLINE __m128d _mm_hadd_pd(__m128d a, __m128d b) { __m128d r = {a[0] + a[1], b[0] + b[1]}; return r; }
SHIM_INLINE __m128d _mm_unpackhi_pd(__m128d a, __m128d b) { __m128d r = {a[1], b[1]}; return r; }
SHIM_INLINE __m128d _mm_shuffle_pd(__m128d a, __m128d b, const int imm) {
    __m128d r = {a[imm & 1], b[(imm >> 1) & 1]};
    return r;
}
SHIM_INLINE __m128d _mm_cmp_pd(__m128d a, __m128d b, const int pred) {
    __shim_m128i m;
    for (int i = 0; i < 2; i++) {
        const int t = pred == _CMP_LT_OQ ? (a[i] < b[i]) : pred == _CMP_GE_OQ ? (a[i] >= b[i]) : 0;
        m[i] = t ? -1LL : 0LL;
    }
    return (__m128d)m;
}
SHIM_INLINE __m128d _mm_blendv_pd(__m128d a, __m128d b, __m128d mask) {
    const __shim_m128i m = (__shim_m128i)mask;
    __m128d r = {m[0] < 0 ? b[0] : a[0], m[1] < 0 ? b[1] : a[1]};
    return r;
}

#undef SHIM_INLINE
#endif
