/*
 * fcs_mlp.h -- the learned surrogate of the GB300 chemistry library.
 *
 * No counterpart in the reference: FastChemistrySolver integrates every
 * cell with Rodas/Rosenbrock/Seulex.  This adds a small MLP ensemble that
 * predicts a cell's state after the CFD step and its next initial sub-step,
 * and a gate that accepts a prediction only when the ensemble members agree
 * and the elements are conserved; every other cell, and a fixed audit
 * fraction of the accepted ones, is integrated by the plain method.
 *
 * Network: n_in -> depth hidden layers of `width` with GELU -> n_out.  BF16
 * operands on the sm_103a tensor cores (tcgen05, TMEM accumulators, TMA),
 * FP32 accumulation, FP32 master weights and Adam, all in the library's own
 * kernels.  Inputs are affine-normalised and outputs de-normalised with the
 * vectors set by fcs_mlp_set_normalization.
 *
 * Parameter layout (FP32, per member): for each layer l = 0..depth, the
 * weight matrix W_l[out][in] row-major, then the bias b_l[out].
 */
#ifndef FCS_MLP_H
#define FCS_MLP_H

#include <stdint.h>
#include "fcs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fcs_mlp fcs_mlp;

typedef struct fcs_mlp_shape {
    int32_t n_in;      /* <= 256 */
    int32_t n_out;     /* <= 256 */
    int32_t width;     /* 256 */
    int32_t depth;     /* hidden layers, 1..8 */
    int32_t members;   /* ensemble size, 1..8 */
} fcs_mlp_shape;

typedef struct fcs_mlp_train_options {
    int32_t epochs;
    int32_t batch;           /* multiple of 128 */
    double lr;               /* Adam step size (cosine-decayed to lr_final) */
    double lr_final;
    double beta1, beta2, eps;
    uint64_t seed;           /* epoch shuffles (member m uses seed + m) */
} fcs_mlp_train_options;

/* Create an ensemble with He-initialised weights (seeded, member m uses
 * seed + m) and identity normalisation. */
fcs_status fcs_mlp_create(fcs_mlp** out, int device, const fcs_mlp_shape* shape, uint64_t seed);
fcs_status fcs_mlp_destroy(fcs_mlp* mlp);
const char* fcs_mlp_last_error(const fcs_mlp* mlp);
fcs_status fcs_mlp_get_shape(const fcs_mlp* mlp, fcs_mlp_shape* shape);
fcs_status fcs_mlp_param_count(const fcs_mlp* mlp, int64_t* count);
fcs_status fcs_mlp_default_train_options(fcs_mlp_train_options* o);

fcs_status fcs_mlp_set_params(fcs_mlp* mlp, int32_t member, const float* params);
fcs_status fcs_mlp_get_params(const fcs_mlp* mlp, int32_t member, float* params);
/* x_norm = (x - in_mean) / in_std;  y = y_norm * out_std + out_mean */
fcs_status fcs_mlp_set_normalization(fcs_mlp* mlp, const float* in_mean, const float* in_std,
                                     const float* out_mean, const float* out_std);
fcs_status fcs_mlp_get_normalization(const fcs_mlp* mlp, float* in_mean, float* in_std,
                                     float* out_mean, float* out_std);

/* y[n][n_out] = member's network at x[n][n_in] (raw units, host or device
 * pointers per flags = FCS_PTR_DEVICE). */
fcs_status fcs_mlp_forward(fcs_mlp* mlp, int32_t member, int64_t n, const float* x, float* y, int32_t flags);

/* One forward + backward pass of `member` on a batch (n a multiple of 128):
 * loss = mean over samples and outputs of (y_norm - target_norm)^2, and its
 * gradient with respect to every parameter (layout of the parameters).
 * Nothing is updated.  Host pointers. */
fcs_status fcs_mlp_gradients(fcs_mlp* mlp, int32_t member, int64_t n, const float* x, const float* target,
                             float* loss, float* grads);

/* Train every member on the same samples (x[n][n_in], target[n][n_out], raw
 * units, host pointers) with Adam; epoch_loss[member * epochs + e] gets the
 * mean training loss of each epoch (may be NULL). */
fcs_status fcs_mlp_train(fcs_mlp* mlp, int64_t n, const float* x, const float* target,
                         const fcs_mlp_train_options* opts, float* epoch_loss);

fcs_status fcs_mlp_save(const fcs_mlp* mlp, const char* path);
fcs_status fcs_mlp_load(fcs_mlp** out, int device, const char* path);

/* ---- the gate: surrogate first, plain method for what it does not accept ----
 *
 * The surrogate attached to a chemistry context has n_in = Ns + 3 inputs
 * (T, ln p, ln delta_t, Y_0 .. Y_{Ns-1}) and n_out = Ns + 2 outputs
 * (T1 - T, Y1_0 - max(Y_0, 0) .. Y1_{Ns-1} - max(Y_{Ns-1}, 0), ln sub_delta_t1),
 * all in raw units (the network's normalisation takes care of the scales).
 * A cell's prediction (the ensemble mean) is accepted when
 *   - every member's T1 is within T_rel * T of the mean,
 *   - every member's Y1_i is within Y_abs of the mean, for every species,
 *   - no predicted Y1_i is below -Y_abs,
 *   - every element's mass fraction sum_i a_ei W_e (Y1_i - Y_i) / W_i changes
 *     by at most element_abs,
 *   - and everything is finite.
 * Accepted cells take the prediction (Y clamped at 0, RR from it, the
 * predicted sub-step capped as the plain method caps it).  Rejected cells
 * are integrated by the configured solver, starting from the predicted
 * sub-step when seed_substep is set, in a work queue ordered by predicted
 * step count (delta_t / predicted sub-step, most expensive first).  A fixed,
 * deterministic audit_fraction of the accepted cells (chosen by a hash of the
 * cell index) is integrated as well and keeps the plain result; the largest
 * surrogate error seen on them is reported.
 */
typedef struct fcs_gate_options {
    double T_rel;           /* default 1e-3 (the method's target accuracy in T) */
    double Y_abs;           /* default 1e-6 (the method's target accuracy in Y_i) */
    double element_abs;     /* default 1e-6 */
    double audit_fraction;  /* default 0.02 */
    int32_t seed_substep;   /* default 1 */
    int32_t reserved;
} fcs_gate_options;

typedef struct fcs_gate_stats {
    int64_t cells_active;       /* T > Treact */
    int64_t cells_accepted;     /* took the surrogate's prediction (audited ones excluded) */
    int64_t cells_fallback;     /* rejected by the gate and integrated */
    int64_t cells_audited;      /* accepted, integrated anyway, plain result kept */
    double audit_max_rel_T;     /* max |T_sur - T| / T over audited cells */
    double audit_max_abs_Y;     /* max |Y_sur,i - Y_i| over audited cells and species */
    double surrogate_ms;        /* features + ensemble + gate + queue */
    double integrate_ms;        /* the plain method on rejected and audited cells */
} fcs_gate_stats;

fcs_status fcs_gate_default_options(fcs_gate_options* o);
/* Attach (or with mlp == NULL detach) a surrogate to ctx.  composition is
 * [Ns][n_elements] atom counts, element_mass [n_elements] (kg/kmol);
 * n_elements <= 8.  The ensemble stays owned by the caller and must outlive
 * its use by ctx. */
fcs_status fcs_surrogate_attach(fcs_ctx* ctx, fcs_mlp* mlp, int32_t n_elements, const double* composition,
                                const double* element_mass, const fcs_gate_options* opts);
/* fcs_integrate with the gate in front (same arguments and results). */
fcs_status fcs_integrate_gated(fcs_ctx* ctx, int64_t n_cells, double delta_t, const double* p, const double* rho0,
                               double* T, double* Y, double* sub_delta_t, double* RR, int32_t* cell_status,
                               fcs_step_stats* stats, double* delta_t_min, int32_t flags, fcs_gate_stats* gstats);

#ifdef __cplusplus
}
#endif
#endif /* FCS_MLP_H */
