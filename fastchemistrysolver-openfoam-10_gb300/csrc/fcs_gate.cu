// fcs_gate.cu -- fcs_integrate_gated: the surrogate ensemble in front of the
// plain integrator (include/fcs_mlp.h).  No counterpart in the reference.
//
// One call, all on the context's stream and without host round trips
// between the phases:
//   classify_kernel      T <= Treact cells: RR = 0, status skipped (as fcs_integrate)
//   features_kernel      x[c] = (T, ln p, ln dt, Y_0..Y_{Ns-1})
//   ensemble forward     members x tensor-core MLP (fcs_mlp.cu)
//   gate_kernel          accept -> write the prediction; reject / audit -> queue bin
//   queue_kernel         work queue ordered by predicted step count, most expensive first
//   integrate_kernel     the plain method on the queue (length read on the device)
//   audit_kernel         surrogate vs plain result on the audited cells
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fcs_mlp.h"
#include "fcs_ctx.h"
#include "fcs_mlp_internal.h"

using namespace fcs;

namespace fcs {

constexpr int kMaxElements = 8;
// gate counters: the binned work-queue counters (QC_*), QC_AUX counting audit records
// gate statistics (unsigned long long): accepted, fallback, audited, max rel T bits, max abs Y bits
enum { GS_ACCEPTED = 0, GS_FALLBACK, GS_AUDITED, GS_RELT, GS_ABSY, GS_ACTIVE, GS_COUNT };

struct GateState {
    fcs_mlp* mlp = nullptr;
    fcs_gate_options opt{};
    int ne = 0;
    DBuf<double> factor;              // [Ns][ne]: a_ei * W_e / W_i
    DBuf<float> x, y;                 // features [nc][nIn], predictions [E][nc][nOut]
    DBuf<int> order, bin, counters, auditCell;
    DBuf<double> auditPred;           // [cap][Ns+1]: predicted Y then T
    DBuf<unsigned long long> gstats;
};

void gate_release(fcs_ctx* ctx) {
    if (!ctx || !ctx->gate) return;
    GateState* g = ctx->gate;
    g->factor.release(); g->x.release(); g->y.release(); g->order.release(); g->bin.release();
    g->counters.release(); g->auditCell.release(); g->auditPred.release(); g->gstats.release();
    delete g;
    ctx->gate = nullptr;
}

__device__ __forceinline__ unsigned long long pos_bits(double v) {
    return static_cast<unsigned long long>(__double_as_longlong(v));
}

__global__ void features_kernel(long long nc, int ns, int nIn, const double* __restrict__ T,
                                const double* __restrict__ p, const double* __restrict__ Y, double dt,
                                float* __restrict__ x) {
    const long long total = nc * nIn;
    const float ldt = (float)log(dt);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long c = i % nc;
        const int k = (int)(i / nc);
        float v;
        if (k == 0) v = (float)T[c];
        else if (k == 1) v = (float)log(p[c]);
        else if (k == 2) v = ldt;
        else v = (float)Y[(size_t)(k - 3) * nc + c];
        x[c * nIn + k] = v;
    }
}

struct GateArgs {
    long long nc;
    int ns, E, nOut, ne;
    double dt, Treact, dtChemMax;
    double Trel, Yabs, elAbs;
    unsigned int auditThreshold;   // of 2^32
    int seedSub, auditCap;
    const float* y;                // [E][nc][nOut]
    const double* factor;          // [Ns][ne]
    const double* rho0;
    double* T;
    double* Y;
    double* sub;
    double* RR;
    int* status;
    int* bin;
    const int* attempts;           // per cell: attempts of the previous integration of this batch
    int attemptsValid;             // attempts[] is valid: bins by it, as the plain method's queue
    int* counters;
    int* auditCell;
    double* auditPred;
    unsigned long long* gstats;
    unsigned long long* dtMinBits;
};

__device__ __forceinline__ unsigned int cell_hash(unsigned long long c) {
    unsigned long long z = c + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (unsigned int)((z ^ (z >> 31)) >> 32);
}

// One warp per cell.
__global__ void __launch_bounds__(256) gate_kernel(const GateArgs a) {
    const int lane = threadIdx.x & 31;
    const long long c = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    if (c >= a.nc) return;
    const double T0 = a.T[c];
    if (!(T0 > a.Treact)) {
        if (lane == 0) a.bin[c] = -1;
        return;
    }
    const size_t stride = (size_t)a.nc * a.nOut;
    const float* yc = a.y + (size_t)c * a.nOut;
    // T and the sub-step (every lane reads the same values)
    double mT = 0, mS = 0;
    for (int e = 0; e < a.E; e++) {
        mT += yc[e * stride];
        mS += yc[e * stride + a.nOut - 1];
    }
    mT /= a.E;
    mS /= a.E;
    double sT = 0;
    for (int e = 0; e < a.E; e++) sT = fmax(sT, fabs((double)yc[e * stride] - mT));
    // species
    double sY = 0, minY = 1e300;
    double el[kMaxElements];
    for (int k = 0; k < kMaxElements; k++) el[k] = 0;
    bool finite = isfinite(mT) && isfinite(mS);
    for (int i = lane; i < a.ns; i += 32) {
        double m = 0;
        for (int e = 0; e < a.E; e++) m += yc[e * stride + 1 + i];
        m /= a.E;
        double s = 0;
        for (int e = 0; e < a.E; e++) s = fmax(s, fabs((double)yc[e * stride + 1 + i] - m));
        const double dY = m;
        finite = finite && isfinite(dY);
        sY = fmax(sY, s);
        const double Yp = fmax(a.Y[(size_t)i * a.nc + c], 0.0) + dY;
        minY = fmin(minY, Yp);
        for (int k = 0; k < a.ne; k++) el[k] += a.factor[i * a.ne + k] * dY;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sY = fmax(sY, __shfl_xor_sync(0xffffffffu, sY, o));
        minY = fmin(minY, __shfl_xor_sync(0xffffffffu, minY, o));
        for (int k = 0; k < a.ne; k++) el[k] += __shfl_xor_sync(0xffffffffu, el[k], o);
    }
    finite = __all_sync(0xffffffffu, finite);
    double elMax = 0;
    for (int k = 0; k < a.ne; k++) elMax = fmax(elMax, fabs(el[k]));
    const double Tp = T0 + mT;
    const double subP = exp(mS);
    const bool accept = finite && isfinite(Tp) && isfinite(subP) && subP > 0 && sT <= a.Trel * T0 &&
                        sY <= a.Yabs && minY >= -a.Yabs && elMax <= a.elAbs;
    const bool audit = accept && cell_hash((unsigned long long)c) < a.auditThreshold;
    if (lane == 0) atomicAdd(&a.gstats[GS_ACTIVE], 1ull);
    if (accept) {
        // the prediction: written to the cell (accepted) or to the audit record
        int slot = -1;
        if (audit) {
            if (lane == 0) slot = atomicAdd(&a.counters[QC_AUX], 1);
            slot = __shfl_sync(0xffffffffu, slot, 0);
            if (slot >= a.auditCap) slot = -2;
        }
        double* rec = slot >= 0 ? a.auditPred + (size_t)slot * (a.ns + 1) : nullptr;
        const double rho0 = a.rho0[c];
        for (int i = lane; i < a.ns; i += 32) {
            const size_t ia = (size_t)i * a.nc + c;
            const double Y0 = a.Y[ia];
            double m = 0;
            for (int e = 0; e < a.E; e++) m += yc[e * stride + 1 + i];
            m /= a.E;
            const double Yn = fmax(fmax(Y0, 0.0) + m, 0.0);
            if (audit) {
                if (rec) rec[i] = Yn;
            } else {
                if (a.RR) a.RR[ia] = (Yn * rho0 - Y0 * rho0) / a.dt;
                a.Y[ia] = Yn;
            }
        }
        if (lane == 0) {
            if (audit) {
                if (rec) {
                    rec[a.ns] = Tp;
                    a.auditCell[slot] = (int)c;
                }
                atomicAdd(&a.gstats[GS_AUDITED], 1ull);
            } else {
                a.T[c] = Tp;
                a.sub[c] = subP < a.dtChemMax ? subP : a.dtChemMax;
                if (a.status) a.status[c] = FCS_CELL_OK;
                a.bin[c] = -1;
                atomicAdd(&a.gstats[GS_ACCEPTED], 1ull);
                atomicMin(a.dtMinBits, pos_bits(subP));
            }
        }
        if (!audit) return;
    } else if (lane == 0) {
        atomicAdd(&a.gstats[GS_FALLBACK], 1ull);
    }
    if (lane == 0) {
        // the cell's cost -> bin (0: cheapest): its attempts in the previous
        // integration of this batch when the context holds them, else the
        // step count predicted from its sub-step
        double sub = a.sub[c];
        if (a.seedSub && isfinite(subP) && subP > 0) {
            sub = fmin(fmax(subP, 1e-14), a.dt);
            a.sub[c] = sub;
        }
        int b;
        if (a.attemptsValid) {
            b = attempt_bin(a.attempts[c]);
        } else {
            const double steps = a.dt / fmax(sub, 1e-300);
            b = steps > 1 ? (int)log2(steps) : 0;
            b = b < 0 ? 0 : (b >= kQueueBins ? kQueueBins - 1 : b);
        }
        a.bin[c] = b;
        atomicAdd(&a.counters[QC_BINS + b], 1);
    }
}

// One warp per audited cell: surrogate prediction vs the plain result.
__global__ void audit_kernel(int ns, long long nc, int cap, const int* counters, const int* __restrict__ cell,
                             const double* __restrict__ pred, const double* __restrict__ T, const double* __restrict__ Y,
                             unsigned long long* gstats) {
    const int lane = threadIdx.x & 31;
    const long long k = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int n = min(counters[QC_AUX], cap);
    if (k >= n) return;
    const long long c = cell[k];
    const double* rec = pred + (size_t)k * (ns + 1);
    double dy = 0;
    for (int i = lane; i < ns; i += 32) dy = fmax(dy, fabs(rec[i] - Y[(size_t)i * nc + c]));
    for (int o = 16; o > 0; o >>= 1) dy = fmax(dy, __shfl_xor_sync(0xffffffffu, dy, o));
    if (lane == 0) {
        const double dT = fabs(rec[ns] - T[c]) / fabs(T[c]);
        atomicMax(&gstats[GS_RELT], pos_bits(isfinite(dT) ? dT : 1e300));
        atomicMax(&gstats[GS_ABSY], pos_bits(isfinite(dy) ? dy : 1e300));
    }
}

}  // namespace fcs

extern "C" fcs_status fcs_gate_default_options(fcs_gate_options* o) {
    if (!o) return FCS_ERR_INVALID;
    // the method's accuracy target: 1e-3 relative in T, 1e-6 absolute in every Y_i
    o->T_rel = 1e-3;
    o->Y_abs = 1e-6;
    o->element_abs = 1e-6;
    o->audit_fraction = 0.02;
    o->seed_substep = 1;
    o->reserved = 0;
    return FCS_OK;
}

extern "C" fcs_status fcs_surrogate_attach(fcs_ctx* ctx, fcs_mlp* mlp, int32_t ne, const double* comp,
                                           const double* emass, const fcs_gate_options* opts) {
    if (!ctx) return FCS_ERR_INVALID;
    if (!mlp) {
        if (fcs_status s = refuse_if_async_pending(ctx)) return s;
        gate_release(ctx);
        return FCS_OK;
    }
    if (!ctx->loaded) return set_err(ctx, FCS_ERR_STATE, "no mechanism loaded");
    if (fcs_status s = refuse_if_async_pending(ctx)) return s;
    const int ns = ctx->M.ns;
    if (mlp_n_in(mlp) != ns + 3 || mlp_n_out(mlp) != ns + 2)
        return set_err(ctx, FCS_ERR_INVALID, "surrogate must have Ns+3 inputs and Ns+2 outputs");
    if (mlp_device(mlp) != ctx->device) return set_err(ctx, FCS_ERR_INVALID, "surrogate lives on another device");
    if (ne < 0 || ne > kMaxElements || (ne > 0 && (!comp || !emass)))
        return set_err(ctx, FCS_ERR_INVALID, "n_elements must be 0..8 with composition and element masses");
    fcs_gate_options o;
    fcs_gate_default_options(&o);
    if (opts) o = *opts;
    if (!(o.T_rel >= 0) || !(o.Y_abs >= 0) || !(o.element_abs >= 0) || !(o.audit_fraction >= 0) || o.audit_fraction > 1)
        return set_err(ctx, FCS_ERR_INVALID, "gate thresholds must be non-negative, audit_fraction in [0, 1]");
    cudaSetDevice(ctx->device);
    gate_release(ctx);
    GateState* g = new GateState();
    g->mlp = mlp;
    g->opt = o;
    g->ne = ne;
    std::vector<double> f((size_t)ns * std::max(ne, 1), 0.0), W(ns);
    CK(cudaMemcpy(W.data(), ctx->M.W, ns * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < ns; i++)
        for (int k = 0; k < ne; k++) f[(size_t)i * ne + k] = comp[(size_t)i * ne + k] * emass[k] / W[i];
    if (g->factor.ensure(f.size()) || g->counters.ensure(QC_COUNT) || g->gstats.ensure(GS_COUNT)) {
        delete g;
        return set_err(ctx, FCS_ERR_NOMEM, "gate allocation failed");
    }
    CK(cudaMemcpy(g->factor.p, f.data(), f.size() * sizeof(double), cudaMemcpyHostToDevice));
    ctx->gate = g;
    return FCS_OK;
}

extern "C" fcs_status fcs_integrate_gated(fcs_ctx* ctx, int64_t nc, double dt, const double* p, const double* rho0,
                                          double* T, double* Y, double* sub, double* RR, int32_t* status,
                                          fcs_step_stats* stats, double* dtMin, int32_t flags, fcs_gate_stats* gst) {
    if (!ctx) return FCS_ERR_INVALID;
    if (!ctx->loaded) return set_err(ctx, FCS_ERR_STATE, "no mechanism loaded");
    GateState* g = ctx->gate;
    if (!g) return set_err(ctx, FCS_ERR_STATE, "no surrogate attached");
    if (fcs_status s = refuse_if_async_pending(ctx)) return s;
    if (nc < 0 || nc > (int64_t)INT32_MAX) return set_err(ctx, FCS_ERR_INVALID, "n_cells out of range");
    if (!p || !rho0 || !T || !Y || !sub) return set_err(ctx, FCS_ERR_INVALID, "null cell array");
    if (!(dt > 0)) return set_err(ctx, FCS_ERR_INVALID, "delta_t must be positive");
    cudaSetDevice(ctx->device);
    const int ns = ctx->M.ns;
    const bool dev = flags & FCS_PTR_DEVICE;
    if (dev) {
        const struct { const void* ptr; const char* name; size_t align; } arrays[] = {
            {p, "p", 8}, {rho0, "rho0", 8}, {T, "T", 8}, {Y, "Y", 8}, {sub, "sub_delta_t", 8},
            {RR, "RR", 8}, {status, "cell_status", 4}};
        for (const auto& a : arrays)
            if (a.ptr)
                if (fcs_status s = check_device_array(ctx, a.ptr, a.name, a.align)) return s;
    }
    cudaStream_t st = ctx->stream;
    const int E = mlp_members(g->mlp), nIn = ns + 3, nOut = ns + 2;
    CellIO io{};
    io.nCells = nc;
    io.deltaT = dt;
    CK(cudaEventRecord(ctx->evc0, st));
    if (dev) {
        io.p = p; io.rho0 = rho0; io.T = T; io.Y = Y; io.subDt = sub; io.RR = RR; io.status = status;
    } else {
        CK(ctx->bp.ensure(nc)); CK(ctx->brho.ensure(nc)); CK(ctx->bT.ensure(nc));
        CK(ctx->bY.ensure((size_t)ns * nc)); CK(ctx->bSub.ensure(nc)); CK(ctx->bStatus.ensure(nc));
        if (RR) CK(ctx->bRR.ensure((size_t)ns * nc));
        CK(cudaMemcpyAsync(ctx->bp.p, p, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->brho.p, rho0, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bT.p, T, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bY.p, Y, (size_t)ns * nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bSub.p, sub, nc * 8, cudaMemcpyHostToDevice, st));
        io.p = ctx->bp.p; io.rho0 = ctx->brho.p; io.T = ctx->bT.p; io.Y = ctx->bY.p;
        io.subDt = ctx->bSub.p; io.RR = RR ? ctx->bRR.p : nullptr; io.status = ctx->bStatus.p;
    }
    const int auditCap = (int)std::min<long long>(nc, (long long)std::ceil(nc * g->opt.audit_fraction * 1.5) + 256);
    CK(ctx->bStats.ensure(ST_COUNT));
    CK(ctx->bMin.ensure(1));
    CK(ctx->bOrder.ensure(std::max<int64_t>(nc, 1)));
    CK(ctx->bHead.ensure(2));
    CK(g->x.ensure((size_t)std::max<int64_t>(nc, 1) * nIn));
    CK(g->y.ensure((size_t)std::max<int64_t>(nc, 1) * nOut * E));
    CK(g->order.ensure(std::max<int64_t>(nc, 1)));
    CK(g->bin.ensure(std::max<int64_t>(nc, 1)));
    CK(g->auditCell.ensure(std::max(auditCap, 1)));
    CK(g->auditPred.ensure((size_t)std::max(auditCap, 1) * (ns + 1)));
    io.stats = ctx->bStats.p;
    io.dtMinBits = ctx->bMin.p;
    // per-cell attempts of the previous integration of a batch of this size
    // (plain or gated) order the fallback queue, as in the plain method
    if (ctx->bAtt.n < (size_t)std::max<int64_t>(nc, 1)) ctx->attN = 0;
    CK(ctx->bAtt.ensure(std::max<int64_t>(nc, 1)));
    io.attempts = ctx->bAtt.p;
    const int attValid = ctx->attN == nc ? 1 : 0;
    CK(cudaMemsetAsync(ctx->bStats.p, 0, ST_COUNT * sizeof(long long), st));
    CK(cudaMemsetAsync(ctx->bMin.p, 0x7f, sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(ctx->bHead.p, 0, 2 * sizeof(int), st));
    CK(cudaMemsetAsync(g->counters.p, 0, QC_COUNT * sizeof(int), st));
    CK(cudaMemsetAsync(g->gstats.p, 0, GS_COUNT * sizeof(unsigned long long), st));
    // the fallback cells run with the plain method's mapping for this batch
    const int group = ctx->opt.mapping ? ctx->opt.mapping : lane_auto(ctx, nc) ? (int)FCS_MAPPING_LANE : [&] {
        const auto key = std::make_tuple(ctx->M.n, (int)ctx->opt.precision, (int)ctx->opt.solver, (int)ctx->opt.jacobian);
        const auto it = ctx->tuned.find(key);
        return it != ctx->tuned.end() ? it->second : default_group(ctx);
    }();
    Shape sh;
    if (!make_shape(ctx, group, true, sh)) return set_err(ctx, FCS_ERR_UNSUPPORTED, "no launch shape for this mapping");
    if (sh.global) {
        const size_t groups = (size_t)sh.lc.grid * (sh.lc.block / sh.lc.group);
        if (ctx->gws.ensure(groups * (size_t)sh.L.bytes) != cudaSuccess)
            return set_err(ctx, FCS_ERR_NOMEM, "global workspace allocation failed");
    }
    if (nc > 0) {
        // T <= Treact: skipped exactly as by fcs_integrate (its queue is not used here)
        CK(launch_classify(io, ns, ctx->opt.T_react, ctx->bOrder.p, ctx->bHead.p + 1, st));
        const int blk = 256;
        const long long fTot = nc * nIn;
        features_kernel<<<(int)std::min<long long>((fTot + blk - 1) / blk, 152LL * 64), blk, 0, st>>>(
            nc, ns, nIn, io.T, io.p, io.Y, dt, g->x.p);
        CK(cudaGetLastError());
        for (int e = 0; e < E; e++) {
            fcs_status s = mlp_forward_device(g->mlp, e, nc, g->x.p, g->y.p + (size_t)e * nc * nOut, st);
            if (s != FCS_OK) return set_err(ctx, s, std::string("surrogate: ") + mlp_message(g->mlp));
        }
        GateArgs a{};
        a.nc = nc; a.ns = ns; a.E = E; a.nOut = nOut; a.ne = g->ne;
        a.dt = dt; a.Treact = ctx->opt.T_react; a.dtChemMax = ctx->opt.delta_t_chem_max;
        a.Trel = g->opt.T_rel; a.Yabs = g->opt.Y_abs; a.elAbs = g->opt.element_abs;
        a.auditThreshold = (unsigned int)std::min(4294967295.0, g->opt.audit_fraction * 4294967296.0);
        a.seedSub = g->opt.seed_substep; a.auditCap = auditCap;
        a.y = g->y.p; a.factor = g->factor.p; a.rho0 = io.rho0; a.T = io.T; a.Y = io.Y; a.sub = io.subDt;
        a.RR = io.RR; a.status = io.status; a.bin = g->bin.p; a.counters = g->counters.p;
        a.attempts = io.attempts; a.attemptsValid = attValid;
        a.auditCell = g->auditCell.p; a.auditPred = g->auditPred.p; a.gstats = g->gstats.p;
        a.dtMinBits = ctx->bMin.p;
        const long long wTot = nc * 32;
        gate_kernel<<<(int)((wTot + 255) / 256), 256, 0, st>>>(a);
        CK(cudaGetLastError());
        CK(launch_queue(nc, g->bin.p, g->counters.p, g->order.p, st));
        CK(cudaEventRecord(ctx->ev0, st));
        WorkQueue q{g->counters.p + QC_HEAD, g->order.p, 0, g->counters.p + QC_LEN};
        const KOpts ko = kopts(ctx->opt);
        CK(launch_integrate(sh.lc, sh.mixed, ctx->M, ko, sh.L, io, q, sh.global ? ctx->gws.p : nullptr, st));
        CK(cudaEventRecord(ctx->ev1, st));
        const long long aTot = (long long)auditCap * 32;
        audit_kernel<<<(int)((aTot + 255) / 256), 256, 0, st>>>(ns, nc, auditCap, g->counters.p, g->auditCell.p,
                                                                 g->auditPred.p, io.T, io.Y, g->gstats.p);
        CK(cudaGetLastError());
        // the integrator recorded the attempts of the cells it ran; accepted
        // cells keep their earlier counts
        ctx->attN = nc;
    } else {
        CK(cudaEventRecord(ctx->ev0, st));
        CK(cudaEventRecord(ctx->ev1, st));
    }
    long long hs[ST_COUNT];
    unsigned long long hg[GS_COUNT], hmin = 0;
    CK(cudaMemcpyAsync(hs, ctx->bStats.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hg, g->gstats.p, sizeof(hg), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&hmin, ctx->bMin.p, sizeof(hmin), cudaMemcpyDeviceToHost, st));
    if (!dev) {
        CK(cudaMemcpyAsync(T, io.T, nc * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Y, io.Y, (size_t)ns * nc * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(sub, io.subDt, nc * 8, cudaMemcpyDeviceToHost, st));
        if (RR) CK(cudaMemcpyAsync(RR, io.RR, (size_t)ns * nc * 8, cudaMemcpyDeviceToHost, st));
        if (status) CK(cudaMemcpyAsync(status, io.status, nc * 4, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaEventRecord(ctx->evc1, st));
    CK(cudaStreamSynchronize(st));
    fcs_status me = mlp_check_errors(g->mlp);
    if (me != FCS_OK) return set_err(ctx, me, std::string("surrogate: ") + mlp_message(g->mlp));
    float ms = 0, cms = 0, pre = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    cudaEventElapsedTime(&cms, ctx->evc0, ctx->evc1);
    cudaGetLastError();  // an elapsed-time query that failed must not leak into the caller's next check
    cudaEventElapsedTime(&pre, ctx->evc0, ctx->ev0);
    if (stats) {
        stats->cells_integrated = hs[ST_CELLS];
        stats->cells_skipped = hs[ST_SKIPPED];
        stats->cells_failed = hs[ST_FAILED];
        stats->attempts = hs[ST_ATTEMPTS];
        stats->accepted = hs[ST_ACCEPTED];
        stats->jacobians = hs[ST_JAC];
        stats->lu_decompositions = hs[ST_LU];
        stats->rhs_evaluations = hs[ST_RHS];
        stats->linear_solves = hs[ST_SOLVES];
        stats->fp64_fallbacks = hs[ST_FALLBACK];
        stats->kernel_ms = ms;
        stats->call_ms = cms;
        stats->mapping = group;
        stats->reserved = 0;
    }
    if (gst) {
        gst->cells_active = (int64_t)hg[GS_ACTIVE];
        gst->cells_accepted = (int64_t)hg[GS_ACCEPTED];
        gst->cells_fallback = (int64_t)hg[GS_FALLBACK];
        gst->cells_audited = (int64_t)hg[GS_AUDITED];
        double rt, ay;
        std::memcpy(&rt, &hg[GS_RELT], 8);
        std::memcpy(&ay, &hg[GS_ABSY], 8);
        gst->audit_max_rel_T = rt;
        gst->audit_max_abs_Y = ay;
        gst->surrogate_ms = pre;
        gst->integrate_ms = ms;
    }
    if (dtMin) {
        double m = 1e15;
        if (hs[ST_CELLS] > 0 || hg[GS_ACCEPTED] > 0) std::memcpy(&m, &hmin, sizeof(m));
        *dtMin = std::min(m, 2 * dt);
    }
    if (hs[ST_FAILED] > 0) return set_err(ctx, FCS_ERR_CELLS, "some cells failed; see cell_status");
    return FCS_OK;
}
