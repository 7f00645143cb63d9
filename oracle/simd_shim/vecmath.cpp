// vecmath.cpp -- the three four-wide vector math routines the reference's
// core calls through glibc's libmvec symbols (src/Reaction/OptReaction.H:58-83:
// vec256_expd, vec256_logd, vec256_powd bound to _ZGVdN4v_exp,
// _ZGVdN4v_log, _ZGVdN4vv_pow), for hosts without libmvec's AVX2 variants.
// TEST INFRASTRUCTURE ONLY: each lane is the scalar libm function.
#include <cmath>

#include "immintrin.h"

// Hidden: the calls from the reference's code in the same library bind here
// at link time, never to another library's vector routine of the same name
// (glibc's AVX2 ones take their arguments in vector registers).
#define SHIM_HIDDEN __attribute__((visibility("hidden")))
SHIM_HIDDEN __m256d fcs_shim_exp4(__m256d x) asm("_ZGVdN4v_exp");
SHIM_HIDDEN __m256d fcs_shim_log4(__m256d x) asm("_ZGVdN4v_log");
SHIM_HIDDEN __m256d fcs_shim_pow4(__m256d x, __m256d y) asm("_ZGVdN4vv_pow");

__m256d fcs_shim_exp4(__m256d x) {
    __m256d r;
    for (int i = 0; i < 4; i++) r[i] = std::exp(x[i]);
    return r;
}

__m256d fcs_shim_log4(__m256d x) {
    __m256d r;
    for (int i = 0; i < 4; i++) r[i] = std::log(x[i]);
    return r;
}

__m256d fcs_shim_pow4(__m256d x, __m256d y) {
    __m256d r;
    for (int i = 0; i < 4; i++) r[i] = std::pow(x[i], y[i]);
    return r;
}
