// fcs_capi.cu -- the C ABI of libfcs_cuda.so (include/fcs.h): context and
// device-memory management, mechanism packing, launch-shape selection
// (autotuner) and the batched integrate / rhs / jacobian / rates entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/fcs.h"
#include "fcs_device.cuh"
#include "fcs_internal.h"
#include "fcs_lane_layout.h"
#include "fcs_launch.h"
#include "fcs_ctx.h"

using namespace fcs;


fcs_status fcs::set_err(fcs_ctx* c, fcs_status s, const std::string& m) {
    if (c) c->err = m;
    return s;
}

fcs_status fcs::cuda_err(fcs_ctx* c, cudaError_t e, const char* where) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // not sticky: the context stays usable
        return set_err(c, FCS_ERR_NOMEM, std::string(where) + ": " + cudaGetErrorString(e));
    }
    return set_err(c, FCS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

fcs_status fcs::refuse_if_async_pending(fcs_ctx* ctx) {
    if (ctx && ctx->asyncPending)
        return set_err(ctx, FCS_ERR_STATE, "a step from fcs_integrate_async is in flight: call fcs_sync first");
    return FCS_OK;
}

fcs_status fcs::check_device_array(fcs_ctx* ctx, const void* ptr, const char* name, size_t align) {
    if (reinterpret_cast<uintptr_t>(ptr) % align != 0)
        return set_err(ctx, FCS_ERR_INVALID, std::string(name) + " is not aligned");
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, FCS_ERR_INVALID, std::string(name) + " is not a device pointer");
    }
    const bool ok = (a.type == cudaMemoryTypeDevice && a.device == ctx->device) || a.type == cudaMemoryTypeManaged;
    if (!ok)
        return set_err(ctx, FCS_ERR_INVALID,
                       std::string(name) + " must be device memory of the context's device (without "
                                           "FCS_PTR_DEVICE the entry points take host arrays)");
    return FCS_OK;
}

namespace {
std::atomic<int> g_injected_alloc_failures{0};
}

bool fcs::take_injected_alloc_failure() {
    int k = g_injected_alloc_failures.load();
    while (k > 0)
        if (g_injected_alloc_failures.compare_exchange_weak(k, k - 1)) return true;
    return false;
}

extern "C" fcs_status fcs_test_fail_allocations(int32_t count) {
    if (count < 0) return FCS_ERR_INVALID;
    g_injected_alloc_failures.store(count);
    return FCS_OK;
}


extern "C" const char* fcs_version(void) { return "fcs-gb300 1.0 (sm_103a)"; }

extern "C" fcs_status fcs_default_options(fcs_options* o) {
    if (!o) return FCS_ERR_INVALID;
    o->solver = FCS_SOLVER_RODAS34;
    o->jacobian = FCS_JACOBIAN_EXACT;
    o->precision = FCS_PRECISION_FP64;
    o->mapping = FCS_MAPPING_AUTO;
    o->abs_tol = 1e-8;
    o->rel_tol = 1e-4;
    o->max_steps = 10000;
    o->max_rejects = 1000;
    o->T_react = 0.0;
    o->delta_t_chem_max = 1e300;
    return FCS_OK;
}

extern "C" fcs_status fcs_create(fcs_ctx** out, int device) {
    if (!out) return FCS_ERR_INVALID;
    *out = nullptr;
    fcs_ctx* ctx = new fcs_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete ctx; return FCS_ERR_CUDA; }
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    ctx->numSMs = v;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    ctx->maxSmemPerBlock = (size_t)v;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        cudaEventCreate(&ctx->evc0) != cudaSuccess || cudaEventCreate(&ctx->evc1) != cudaSuccess) {
        delete ctx;
        return FCS_ERR_CUDA;
    }
    fcs_default_options(&ctx->opt);
    *out = ctx;
    return FCS_OK;
}

extern "C" fcs_status fcs_destroy(fcs_ctx* ctx) {
    if (!ctx) return FCS_OK;
    cudaSetDevice(ctx->device);
    // a step from fcs_integrate_async may still run on the caller's stream
    if (ctx->asyncPending && ctx->evAsync) cudaEventSynchronize(ctx->evAsync);
    cudaStreamSynchronize(ctx->stream);
    gate_release(ctx);
    for (DBuf<double>* b : {&ctx->dW, &ctx->dInvW, &ctx->dTc, &ctx->dCoef, &ctx->dEff, &ctx->dPlogRow,
                            &ctx->dPlogTa, &ctx->dHf, &ctx->dFo, &ctx->bp, &ctx->brho, &ctx->bT, &ctx->bY,
                            &ctx->bSub, &ctx->bRR, &ctx->bDt, &ctx->bOut, &ctx->bJ, &ctx->bQ})
        b->release();
    ctx->dRx.release();
    ctx->dPlogOff.release(); ctx->dIncOff.release(); ctx->dInc.release(); ctx->dTbInc.release();
    ctx->bStatus.release(); ctx->bOrder.release(); ctx->bHead.release();
    ctx->bStats.release(); ctx->bMin.release(); ctx->gws.release(); ctx->bBin.release(); ctx->bAtt.release();
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    if (ctx->hStats) cudaFreeHost(ctx->hStats);
    if (ctx->evAsync) cudaEventDestroy(ctx->evAsync);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->evc0) cudaEventDestroy(ctx->evc0);
    if (ctx->evc1) cudaEventDestroy(ctx->evc1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return FCS_OK;
}

extern "C" const char* fcs_last_error_string(const fcs_ctx* ctx) {
    return ctx ? ctx->err.c_str() : "null context";
}

extern "C" fcs_status fcs_set_options(fcs_ctx* ctx, const fcs_options* o) {
    if (!ctx || !o) return FCS_ERR_INVALID;
    if (o->solver < 0 || o->solver > 4) return set_err(ctx, FCS_ERR_INVALID, "solver must be 0..4");
    if (o->jacobian < 0 || o->jacobian > 1) return set_err(ctx, FCS_ERR_INVALID, "jacobian must be exact or fast");
    if (o->precision < 0 || o->precision > 1) return set_err(ctx, FCS_ERR_INVALID, "precision must be fp64 or mixed");
    if (!(o->abs_tol > 0) || !(o->rel_tol > 0)) return set_err(ctx, FCS_ERR_INVALID, "tolerances must be positive");
    if (o->max_steps <= 0 || o->max_rejects <= 0) return set_err(ctx, FCS_ERR_INVALID, "maxSteps must be positive");
    const int m = o->mapping;
    if (m != 0 && m != 1 && m != 32 && m != 64 && m != 128 && m != 256)
        return set_err(ctx, FCS_ERR_INVALID, "mapping must be auto, lane (1), 32, 64, 128 or 256");
    ctx->opt = *o;
    return FCS_OK;
}

extern "C" fcs_status fcs_formation_enthalpy(fcs_ctx* ctx, double* hf) {
    if (!ctx || !hf) return FCS_ERR_INVALID;
    if (!ctx->loaded) return set_err(ctx, FCS_ERR_STATE, "no mechanism loaded");
    if (fcs_status s = refuse_if_async_pending(ctx)) return s;
    cudaSetDevice(ctx->device);
    CK(cudaMemcpy(hf, ctx->M.hf, ctx->M.ns * sizeof(double), cudaMemcpyDeviceToHost));
    return FCS_OK;
}

extern "C" fcs_status fcs_mechanism_size(const fcs_ctx* ctx, int32_t* ns, int32_t* nr) {
    if (!ctx || !ctx->loaded) return FCS_ERR_STATE;
    if (ns) *ns = ctx->M.ns;
    if (nr) *nr = ctx->M.nr;
    return FCS_OK;
}

// ------------------------------------------------------------------------
// mechanism packing: type-block order of OptReaction::readInfo
// (OptReaction.C:448-1175), species incidence lists in reaction order.

extern "C" fcs_status fcs_load_mechanism(fcs_ctx* ctx, const fcs_mechanism_desc* d) {
    if (!ctx || !d) return FCS_ERR_INVALID;
    if (fcs_status s = refuse_if_async_pending(ctx)) return s;
    const int ns = d->n_species, nr = d->n_reactions;
    if (ns < 1 || nr < 0) return set_err(ctx, FCS_ERR_INVALID, "bad species/reaction count");
    if (ns > 255) return set_err(ctx, FCS_ERR_UNSUPPORTED, "the GPU path handles up to 255 species");
    if (!d->W || !d->T_low || !d->T_high || !d->T_common || !d->high_coeffs || !d->low_coeffs)
        return set_err(ctx, FCS_ERR_INVALID, "missing species arrays");
    if (nr > 0 && (!d->type || !d->reversible || !d->lhs_offset || !d->lhs_species || !d->rhs_offset ||
                   !d->rhs_species || !d->arrhenius))
        return set_err(ctx, FCS_ERR_INVALID, "missing reaction arrays");
    std::vector<int> order;
    // type blocks: T-independent Arrhenius, Arrhenius, non-equilibrium,
    // non-equilibrium third body (OptReaction.C:610-700), third body, fall-off
    // (Lindemann, Troe, SRI: OptReaction.C:746-917), PLOG
    static const int kBlocks[] = {FCS_RXN_ARRHENIUS, FCS_RXN_ARRHENIUS, FCS_RXN_NONEQ, FCS_RXN_NONEQ_THIRD_BODY,
                                  FCS_RXN_THIRD_BODY, FCS_RXN_LINDEMANN_FALLOFF, FCS_RXN_TROE_FALLOFF,
                                  FCS_RXN_SRI_FALLOFF, FCS_RXN_PLOG};
    for (int pass = 0; pass < 9; pass++) {
        for (int r = 0; r < nr; r++) {
            const int t = d->type[r];
            if (t != kBlocks[pass]) continue;
            const bool tind = d->arrhenius[3 * r + 1] == 0 && d->arrhenius[3 * r + 2] == 0;
            if (t == FCS_RXN_ARRHENIUS && tind != (pass == 0)) continue;
            order.push_back(r);
        }
    }
    if ((int)order.size() != nr)
        return set_err(ctx, FCS_ERR_UNSUPPORTED,
                       "reaction types other than (ir)reversible Arrhenius, ThirdBodyArrhenius, "
                       "ArrheniusLindemann/Troe/SRIFallOff, ArrheniusPLOG and nonEquilibriumReversible"
                       "(ThirdBody)Arrhenius are not supported by the GPU path");
    std::vector<double> W(ns), invW(ns), Tc(ns), coef(16 * (size_t)ns, 0.0), hf(ns);
    double TlowMin = 1e10, ThighMax = 1, TcMin = 1e10, TcMax = 0;
    for (int i = 0; i < ns; i++) {
        if (!(d->W[i] > 0)) return set_err(ctx, FCS_ERR_INVALID, "molecular weight must be positive");
        W[i] = d->W[i];
        invW[i] = 1.0 / d->W[i];
        Tc[i] = d->T_common[i];
        for (int j = 0; j < 7; j++) {
            coef[16 * i + j] = d->low_coeffs[7 * i + j];
            coef[16 * i + 8 + j] = d->high_coeffs[7 * i + j];
        }
        TlowMin = std::min(TlowMin, d->T_low[i]);
        ThighMax = std::max(ThighMax, d->T_high[i]);
        TcMin = std::min(TcMin, d->T_common[i]);
        TcMax = std::max(TcMax, d->T_common[i]);
        // formation enthalpy at Tstd = 298.15 K (janaf Hf), J/kg
        const double* a = (298.15 < d->T_common[i]) ? &d->low_coeffs[7 * i] : &d->high_coeffs[7 * i];
        const double T = 298.15;
        hf[i] = kRu * invW[i] *
                (((((a[4] / 5 * T + a[3] / 4) * T + a[2] / 3) * T + a[1] / 2) * T + a[0]) * T + a[5]);
    }
    std::vector<RxnInfo> rx(std::max(nr, 1));
    std::vector<double> eff;
    std::vector<int> plogOff{0};
    std::vector<double> plogRow, plogTa, fo;
    std::vector<std::vector<int>> inc(ns);
    std::vector<int> tbInc;
    int nTB = 0, nPlog = 0;
    for (int k = 0; k < nr; k++) {
        const int r = order[k];
        RxnInfo& x = rx[k];
        std::memset(&x, 0, sizeof(x));
        x.A = d->arrhenius[3 * r];
        x.beta = d->arrhenius[3 * r + 1];
        x.Ta = d->arrhenius[3 * r + 2];
        const int l0 = d->lhs_offset[r], l1 = d->lhs_offset[r + 1];
        const int r0 = d->rhs_offset[r], r1 = d->rhs_offset[r + 1];
        if (l1 - l0 < 1 || r1 - r0 < 1)
            return set_err(ctx, FCS_ERR_INVALID, "reaction without reactants or products");
        if (l1 - l0 > kMaxL || r1 - r0 > kMaxR)
            return set_err(ctx, FCS_ERR_UNSUPPORTED, "reactions with more than 4 reactants or 8 products "
                                                     "are not supported by the GPU path");
        x.nl = int8_t(l1 - l0);
        x.nr = int8_t(r1 - r0);
        for (int q = 0; q < x.nl; q++) {
            const int sp = d->lhs_species[l0 + q];
            if (sp < 0 || sp >= ns) return set_err(ctx, FCS_ERR_INVALID, "species index out of range");
            x.sl[q] = uint8_t(sp);
            inc[sp].push_back(k << 1);
        }
        for (int q = 0; q < x.nr; q++) {
            const int sp = d->rhs_species[r0 + q];
            if (sp < 0 || sp >= ns) return set_err(ctx, FCS_ERR_INVALID, "species index out of range");
            x.sr[q] = uint8_t(sp);
            inc[sp].push_back((k << 1) | 1);
        }
        const bool noneq = d->type[r] == FCS_RXN_NONEQ || d->type[r] == FCS_RXN_NONEQ_THIRD_BODY;
        x.rev = noneq ? 2 : d->reversible[r] ? 1 : 0;
        x.kind = int8_t(d->type[r]);
        x.dnu = x.nr - x.nl;
        x.tind = (x.beta == 0 && x.Ta == 0) ? 1 : 0;
        x.tb = -1;
        x.plog = -1;
        x.fo = -1;
        x.nq = -1;
        const bool falloff = d->type[r] >= FCS_RXN_LINDEMANN_FALLOFF && d->type[r] <= FCS_RXN_SRI_FALLOFF;
        if (falloff) {
            if (!d->arrhenius2) return set_err(ctx, FCS_ERR_INVALID, "fall-off reaction without kInf (arrhenius2)");
            if (d->type[r] != FCS_RXN_LINDEMANN_FALLOFF && !d->falloff_params)
                return set_err(ctx, FCS_ERR_INVALID, "Troe/SRI reaction without falloff_params");
            x.fo = (int)(fo.size() / 8);
            for (int q = 0; q < 3; q++) fo.push_back(d->arrhenius2[3 * (size_t)r + q]);
            for (int q = 0; q < 5; q++) fo.push_back(d->falloff_params ? d->falloff_params[5 * (size_t)r + q] : 0.0);
        }
        if (noneq) {
            // the reverse rate's own Arrhenius (OptReaction.C:628-630, 663-665)
            if (!d->arrhenius2)
                return set_err(ctx, FCS_ERR_INVALID, "non-equilibrium reaction without a reverse rate (arrhenius2)");
            x.nq = (int)(fo.size() / 8);
            for (int q = 0; q < 3; q++) fo.push_back(d->arrhenius2[3 * (size_t)r + q]);
            for (int q = 0; q < 5; q++) fo.push_back(0.0);
        }
        if (d->type[r] == FCS_RXN_THIRD_BODY || d->type[r] == FCS_RXN_NONEQ_THIRD_BODY || falloff) {
            if (!d->efficiencies) return set_err(ctx, FCS_ERR_INVALID, "third-body reaction without efficiencies");
            for (int s = 0; s < ns; s++) eff.push_back(d->efficiencies[(size_t)r * ns + s]);
            x.tb = nTB++;
            for (int q = 0; q < x.nl; q++) tbInc.push_back((int(x.sl[q]) << 16) | (x.tb << 1));
            for (int q = 0; q < x.nr; q++) tbInc.push_back((int(x.sr[q]) << 16) | (x.tb << 1) | 1);
        }
        if (d->type[r] == FCS_RXN_PLOG) {
            if (!d->plog_offset || !d->plog_table) return set_err(ctx, FCS_ERR_INVALID, "PLOG reaction without table");
            const int q0 = d->plog_offset[r], q1 = d->plog_offset[r + 1];
            if (q1 - q0 < 1) return set_err(ctx, FCS_ERR_INVALID, "empty PLOG table");
            for (int q = q0; q < q1; q++) {
                const double* row = &d->plog_table[4 * (size_t)q];
                if (!(row[0] > 0) || !(row[1] > 0)) return set_err(ctx, FCS_ERR_INVALID, "PLOG p and A must be positive");
                plogRow.push_back(row[0]);
                plogRow.push_back(std::log(row[0]));
                plogRow.push_back(std::log(row[1]));
                plogRow.push_back(row[2]);
                plogTa.push_back(row[3]);
            }
            plogOff.push_back(plogOff.back() + (q1 - q0));
            x.plog = nPlog++;
        }
    }
    std::vector<int> incOff(ns + 1, 0), incv;
    for (int i = 0; i < ns; i++) {
        incOff[i + 1] = incOff[i] + (int)inc[i].size();
        incv.insert(incv.end(), inc[i].begin(), inc[i].end());
    }
    if (incv.empty()) incv.push_back(0);
    const int nTbInc = (int)tbInc.size();
    if (tbInc.empty()) tbInc.push_back(0);
    if (nTB >= 32768) return set_err(ctx, FCS_ERR_UNSUPPORTED, "too many third-body reactions");
    if (eff.empty()) eff.push_back(0);
    if (plogRow.empty()) { plogRow.assign(4, 0); plogTa.assign(1, 0); }
    if (fo.empty()) fo.assign(8, 0.0);
    cudaSetDevice(ctx->device);
    auto up = [&](auto& buf, const auto& v) -> cudaError_t {
        cudaError_t e = buf.ensure(v.size());
        if (e != cudaSuccess) return e;
        return cudaMemcpy(buf.p, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice);
    };
    CK(up(ctx->dW, W)); CK(up(ctx->dInvW, invW)); CK(up(ctx->dTc, Tc)); CK(up(ctx->dCoef, coef));
    CK(up(ctx->dRx, rx)); CK(up(ctx->dEff, eff)); CK(up(ctx->dPlogOff, plogOff));
    CK(up(ctx->dPlogRow, plogRow)); CK(up(ctx->dPlogTa, plogTa)); CK(up(ctx->dIncOff, incOff));
    CK(up(ctx->dInc, incv)); CK(up(ctx->dHf, hf)); CK(up(ctx->dTbInc, tbInc)); CK(up(ctx->dFo, fo));
    DevMech& M = ctx->M;
    M.ns = ns; M.n = ns + 1; M.nr = nr; M.nTB = nTB; M.nPlog = nPlog;
    M.TlowMin = TlowMin; M.ThighMax = ThighMax; M.TcommonMin = TcMin; M.TcommonMax = TcMax;
    M.W = ctx->dW.p; M.invW = ctx->dInvW.p; M.Tcommon = ctx->dTc.p; M.coef = ctx->dCoef.p;
    M.rx = ctx->dRx.p; M.eff = ctx->dEff.p; M.plogOff = ctx->dPlogOff.p; M.plogRow = ctx->dPlogRow.p;
    M.plogTa = ctx->dPlogTa.p; M.incOff = ctx->dIncOff.p; M.inc = ctx->dInc.p; M.hf = ctx->dHf.p;
    M.nTbInc = nTbInc; M.tbInc = ctx->dTbInc.p;
    M.fo = ctx->dFo.p;
    // the special block: first to last non-equilibrium or fall-off reaction
    // (third-body reactions between them included)
    M.spBegin = 0;
    M.nSp = 0;
    for (int k = 0; k < nr; k++)
        if (rx[k].fo >= 0 || rx[k].nq >= 0) {
            if (M.nSp == 0) M.spBegin = k;
            M.nSp = k + 1 - M.spBegin;
        }
    ctx->loaded = true;
    ctx->tuned.clear();
    if (ctx->gexec) {  // a captured step holds the old mechanism's scalars
        cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
    }
    return FCS_OK;
}

// ------------------------------------------------------------------------
// launch shapes

KOpts fcs::kopts(const fcs_options& o) {
    KOpts k;
    k.solver = o.solver;
    k.jacobian = o.jacobian;
    k.maxSteps = o.max_steps;
    k.maxRejects = o.max_rejects;
    k.absTol = o.abs_tol;
    k.relTol = o.rel_tol;
    k.Treact = o.T_react;
    k.dtChemMax = o.delta_t_chem_max;
    return k;
}

// Lane per cell (FCS_MAPPING_LANE): blocks of 128 threads, three per SM
// (the kernel is compiled for three: 168 registers per thread), a
// global-memory workspace of make_lane_layout(...).words doubles per thread.
// Rosenbrock-family solvers, FP64 or mixed precision.
static bool make_lane_shape(fcs_ctx* ctx, bool integrate, Shape& sh) {
    const fcs_options& o = ctx->opt;
    const bool mixed = o.precision == FCS_PRECISION_MIXED;
    if (!integrate || o.solver == FCS_SOLVER_SEULEX) return false;
    int maxThreads = 0, regs = 0;
    if (integrate_attributes(1, mixed, &maxThreads, &regs) != cudaSuccess) return false;
    constexpr int kBlock = 128;
    if (maxThreads < kBlock) return false;
    const int maxPerSM = std::max(1, std::min(4, 65536 / std::max(1, regs * kBlock)));
    // Three resident blocks (12 warps) per SM by default: on the 53-species
    // field (65,536 cells) 3 blocks ran 5,531 cells/s against 5,311 with 4
    // and 4,970 with 2 -- fewer lanes than cells let the lanes that finish
    // early take the remaining cells.  FCS_LANE_BLOCKS_PER_SM overrides it.
    int perSM = std::min(3, maxPerSM);
    if (const char* e = std::getenv("FCS_LANE_BLOCKS_PER_SM")) {
        const int v = std::atoi(e);
        if (v >= 1) perSM = std::min(maxPerSM, v);
    }
    sh.mixed = mixed;
    sh.global = true;
    sh.lc.group = 1;
    sh.lc.block = kBlock;
    sh.lc.grid = ctx->numSMs * perSM;
    sh.L = SlotLayout{};
    sh.L.bytes = make_lane_layout(ctx->M.ns, ctx->M.nr, ctx->M.nTB, mixed).words * (int)sizeof(double);
    return true;
}

// Build the launch shape for a group size; returns false when impossible.
bool fcs::make_shape(fcs_ctx* ctx, int group, bool integrate, Shape& sh) {
    if (group == FCS_MAPPING_LANE) return make_lane_shape(ctx, integrate, sh);
    const fcs_options& o = ctx->opt;
    const bool mixed = o.precision == FCS_PRECISION_MIXED;
    const bool seulex = integrate && o.solver == FCS_SOLVER_SEULEX;
    sh.mixed = mixed;
    sh.lc.group = group;
    if (ctx->M.n > 256) return false;  // the solves keep <= 256 unknowns per warp lane set
    const size_t smemCap = ctx->maxSmemPerBlock;
    int maxThreads = 0, regs = 0;
    if (integrate_attributes(group, mixed, &maxThreads, &regs) != cudaSuccess) return false;
    // Cells resident per SM for a layout: groups per block (group 32 packs up
    // to 8 cells into a block), blocks per SM by shared memory and registers.
    struct Res { int gpb, perSM; bool global; int cells; };
    auto residency = [&](const SlotLayout& L) {
        Res r;
        r.gpb = 1;
        if (group == 32) r.gpb = (int)std::max<size_t>(1, std::min<size_t>(8, smemCap / (size_t)L.bytes));
        r.global = (size_t)L.bytes > smemCap;
        const int block = group * r.gpb;
        const int bySmem = r.global ? 2 : (int)std::max<size_t>(1, (228 * 1024) / ((size_t)L.bytes * r.gpb + 1024));
        const int byRegs = std::max(1, 65536 / std::max(1, regs * block));
        r.perSM = std::max(1, std::min(bySmem, byRegs));
        r.cells = r.gpb * r.perSM;
        return r;
    };
    // One chunk of reactions unless smaller chunks let more cells reside;
    // then the largest chunk (a multiple of the group size) that does.
    const int nr = std::max(1, ctx->M.nr);
    auto layout = [&](int rc) { return make_layout(ctx->M.ns, ctx->M.nr, ctx->M.nTB, mixed, seulex, rc); };
    sh.L = layout(nr);
    Res res = residency(sh.L);
    if (!res.global && nr > group) {
        const Res best = residency(layout(group));
        if (!best.global && best.cells > res.cells) {
            for (int rc = ((nr - 1) / group) * group; rc >= group; rc -= group) {
                const SlotLayout L = layout(rc);
                const Res r = residency(L);
                if (r.cells == best.cells) { sh.L = L; res = r; break; }
            }
        }
    }
    sh.global = res.global;
    sh.lc.block = group * res.gpb;
    if (sh.lc.block > maxThreads) return false;
    const int perSM = res.perSM;
    sh.lc.grid = ctx->numSMs * perSM;
    return true;
}

fcs_status fcs::ensure_gws(fcs_ctx* ctx, const Shape& sh) {
    if (!sh.global) return FCS_OK;
    const size_t groups = (size_t)sh.lc.grid * (sh.lc.block / sh.lc.group);
    if (ctx->gws.ensure(groups * (size_t)sh.L.bytes) != cudaSuccess)
        return set_err(ctx, FCS_ERR_NOMEM, "global workspace allocation failed");
    return FCS_OK;
}

int fcs::default_group(fcs_ctx* ctx) {
    const int n = ctx->M.n;
    if (n <= 128) return 64;
    return 128;
}

// AUTO chooses the lane mapping for a Rosenbrock-family FP64 step with cells
// enough to occupy most of its lanes (at fewer cells its lanes idle and the
// cell groups, which spread one cell over many threads, are faster).
bool fcs::lane_auto(fcs_ctx* ctx, long long cells) {
    if (ctx->opt.mapping != FCS_MAPPING_AUTO) return false;
    Shape sh;
    if (!make_shape(ctx, FCS_MAPPING_LANE, true, sh)) return false;
    return cells * 4 >= 3LL * sh.lc.grid * sh.lc.block;
}

int fcs::cached_group(fcs_ctx* ctx) {
    if (ctx->opt.mapping) return ctx->opt.mapping;
    const auto it = ctx->tuned.find(
        std::make_tuple(ctx->M.n, (int)ctx->opt.precision, (int)ctx->opt.solver, (int)ctx->opt.jacobian));
    return it != ctx->tuned.end() ? it->second : default_group(ctx);
}

// Autotuner for FCS_MAPPING_AUTO: times every candidate cell-to-thread
// mapping on the first `sample` queued cells, integrated from copies of their
// state (the caller's arrays are not touched), and keeps the fastest for this
// (mechanism size, precision, solver, Jacobian) key.
static int tuned_group(fcs_ctx* ctx, const CellIO& io, int nActive) {
    const auto key = std::make_tuple(ctx->M.n, (int)ctx->opt.precision, (int)ctx->opt.solver, (int)ctx->opt.jacobian);
    auto it = ctx->tuned.find(key);
    if (it != ctx->tuned.end()) return it->second;
    const int fallback = default_group(ctx);
    if (nActive < 2048) return fallback;  // too few cells to time reliably; not cached
    const int ns = ctx->M.ns;
    const long long nc = io.nCells;
    cudaStream_t st = ctx->stream;
    DBuf<double> T, Y, S;
    DBuf<int> stat, head;
    if (T.ensure(nc) || Y.ensure((size_t)ns * nc) || S.ensure(nc) || stat.ensure(nc) || head.ensure(1)) {
        T.release(); Y.release(); S.release(); stat.release(); head.release();
        return fallback;
    }
    const KOpts ko = kopts(ctx->opt);
    int best = fallback;
    float bestMs = 1e30f;
    for (int g : {32, 64, 128, 256}) {
        Shape sh;
        if (!make_shape(ctx, g, true, sh)) continue;
        if (ensure_gws(ctx, sh) != FCS_OK) continue;
        const int groups = sh.lc.grid * (sh.lc.block / g);
        const int sample = std::min(nActive, 2 * groups);
        CellIO sio = io;
        sio.T = T.p; sio.Y = Y.p; sio.subDt = S.p; sio.RR = nullptr; sio.status = stat.p;
        cudaMemcpyAsync(T.p, io.T, nc * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(Y.p, io.Y, (size_t)ns * nc * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(S.p, io.subDt, nc * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemsetAsync(head.p, 0, sizeof(int), st);
        WorkQueue q{head.p, ctx->bOrder.p, sample};
        cudaEventRecord(ctx->ev0, st);
        const cudaError_t e = launch_integrate(sh.lc, sh.mixed, ctx->M, ko, sh.L, sio, q,
                                               sh.global ? ctx->gws.p : nullptr, st);
        cudaEventRecord(ctx->ev1, st);
        if (e != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) continue;
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        const float perCell = ms / sample;
        if (perCell < bestMs) { bestMs = perCell; best = g; }
    }
    T.release(); Y.release(); S.release(); stat.release(); head.release();
    // the statistics of the sample runs are not the caller's
    cudaMemsetAsync(ctx->bStats.p, 0, ST_COUNT * sizeof(long long), st);
    cudaMemsetAsync(ctx->bMin.p, 0x7f, sizeof(unsigned long long), st);
    cudaStreamSynchronize(st);
    ctx->tuned[key] = best;
    return best;
}

// ------------------------------------------------------------------------
// integration

static fcs_status integrate_impl(fcs_ctx* ctx, int64_t nc, double dt, const double* dtc,
                                 const double* p, const double* rho0, double* T, double* Y,
                                 double* sub, double* RR, int32_t* status, fcs_step_stats* stats,
                                 double* dtMin, int32_t flags) {
    if (!ctx) return FCS_ERR_INVALID;
    if (!ctx->loaded) return set_err(ctx, FCS_ERR_STATE, "no mechanism loaded");
    if (fcs_status s = refuse_if_async_pending(ctx)) return s;
    if (nc < 0 || nc > (int64_t)INT32_MAX) return set_err(ctx, FCS_ERR_INVALID, "n_cells out of range");
    if (!p || !rho0 || !T || !Y || !sub) return set_err(ctx, FCS_ERR_INVALID, "null cell array");
    if (!dtc && !(dt > 0)) return set_err(ctx, FCS_ERR_INVALID, "delta_t must be positive");
    cudaSetDevice(ctx->device);
    const int ns = ctx->M.ns;
    const bool dev = flags & FCS_PTR_DEVICE;
    if (dev) {
        const struct { const void* ptr; const char* name; size_t align; } arrays[] = {
            {p, "p", 8}, {rho0, "rho0", 8}, {T, "T", 8}, {Y, "Y", 8}, {sub, "sub_delta_t", 8},
            {RR, "RR", 8}, {status, "cell_status", 4}, {dtc, "delta_t", 8}};
        for (const auto& a : arrays)
            if (a.ptr)
                if (fcs_status s = check_device_array(ctx, a.ptr, a.name, a.align)) return s;
    }
    cudaStream_t st = ctx->stream;
    CellIO io{};
    io.nCells = nc;
    io.deltaT = dt;
    CK(cudaEventRecord(ctx->evc0, st));
    if (dev) {
        io.p = p; io.rho0 = rho0; io.T = T; io.Y = Y; io.subDt = sub; io.RR = RR; io.status = status;
        io.dtPerCell = dtc;
    } else {
        CK(ctx->bp.ensure(nc)); CK(ctx->brho.ensure(nc)); CK(ctx->bT.ensure(nc));
        CK(ctx->bY.ensure((size_t)ns * nc)); CK(ctx->bSub.ensure(nc)); CK(ctx->bStatus.ensure(nc));
        if (RR) CK(ctx->bRR.ensure((size_t)ns * nc));
        if (dtc) CK(ctx->bDt.ensure(nc));
        CK(cudaMemcpyAsync(ctx->bp.p, p, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->brho.p, rho0, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bT.p, T, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bY.p, Y, (size_t)ns * nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bSub.p, sub, nc * 8, cudaMemcpyHostToDevice, st));
        if (dtc) CK(cudaMemcpyAsync(ctx->bDt.p, dtc, nc * 8, cudaMemcpyHostToDevice, st));
        io.p = ctx->bp.p; io.rho0 = ctx->brho.p; io.T = ctx->bT.p; io.Y = ctx->bY.p;
        io.subDt = ctx->bSub.p; io.RR = RR ? ctx->bRR.p : nullptr; io.status = ctx->bStatus.p;
        io.dtPerCell = dtc ? ctx->bDt.p : nullptr;
    }
    const bool sorted = !(flags & FCS_NO_QUEUE_SORT);
    const bool graph = flags & FCS_CUDA_GRAPH;
    if (graph && !dev) return set_err(ctx, FCS_ERR_INVALID, "FCS_CUDA_GRAPH needs FCS_PTR_DEVICE");
    CK(ctx->bStats.ensure(ST_COUNT));
    CK(ctx->bMin.ensure(1));
    CK(ctx->bOrder.ensure(std::max<int64_t>(nc, 1)));
    CK(ctx->bHead.ensure(QC_COUNT));  // head, length and the bin counters of the queue
    if (sorted) CK(ctx->bBin.ensure(std::max<int64_t>(nc, 1)));
    io.stats = ctx->bStats.p;
    io.dtMinBits = ctx->bMin.p;
    // per-cell attempts of the previous call on a batch of this size order the
    // queue (the cells' costs change slowly from one CFD step to the next)
    if (ctx->bAtt.n < (size_t)std::max<int64_t>(nc, 1)) ctx->attN = 0;
    CK(ctx->bAtt.ensure(std::max<int64_t>(nc, 1)));
    io.attempts = ctx->bAtt.p;
    io.attemptsValid = (sorted && ctx->attN == nc) ? 1 : 0;
    const KOpts ko = kopts(ctx->opt);
    // The step's device work: counters, classify (cells with T <= Treact are
    // skipped, transientSolve.H:39, 70-76), the queue ordered by predicted
    // step count, and the persistent integrator reading the queue length on
    // the device.
    auto enqueue_prologue = [&]() -> cudaError_t {
        cudaError_t e;
        if ((e = cudaMemsetAsync(ctx->bStats.p, 0, ST_COUNT * sizeof(long long), st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(ctx->bMin.p, 0x7f, sizeof(unsigned long long), st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(ctx->bHead.p, 0, QC_COUNT * sizeof(int), st)) != cudaSuccess) return e;
        if (!sorted) return launch_classify(io, ns, ctx->opt.T_react, ctx->bOrder.p, ctx->bHead.p + QC_LEN, st);
        if ((e = launch_classify_binned(io, ns, ctx->opt.T_react, ctx->bBin.p, ctx->bHead.p, st)) != cudaSuccess)
            return e;
        return launch_queue(nc, ctx->bBin.p, ctx->bHead.p, ctx->bOrder.p, st);
    };
    long long* hs = ctx->hStats;
    unsigned long long hminv = 0;
    unsigned long long* hmin = &hminv;
    long long hsLocal[ST_COUNT];
    int group = 0;
    if (graph) {
        // one CUDA graph per step shape: replayed while the arrays, sizes and
        // options stay the same, re-captured when any of them changes
        if (!ctx->hStats) CK(cudaMallocHost(&ctx->hStats, (ST_COUNT + 1) * sizeof(long long)));
        hs = ctx->hStats;
        hmin = reinterpret_cast<unsigned long long*>(ctx->hStats + ST_COUNT);
        group = ctx->opt.mapping ? ctx->opt.mapping : lane_auto(ctx, nc) ? (int)FCS_MAPPING_LANE : [&] {
            const auto it = ctx->tuned.find(std::make_tuple(ctx->M.n, (int)ctx->opt.precision, (int)ctx->opt.solver,
                                                            (int)ctx->opt.jacobian));
            return it != ctx->tuned.end() ? it->second : default_group(ctx);
        }();
        Shape sh;
        if (!make_shape(ctx, group, true, sh))
            return set_err(ctx, FCS_ERR_UNSUPPORTED, "no launch shape for this mapping");
        fcs_status s = ensure_gws(ctx, sh);
        if (s != FCS_OK) return s;
        GraphKey key;
        std::memset(&key, 0, sizeof(key));
        key.p = p; key.rho0 = rho0; key.T = T; key.Y = Y; key.sub = sub; key.RR = RR; key.status = status;
        key.dtc = dtc; key.nc = nc; key.dt = dt; key.opt = ctx->opt; key.group = group; key.sorted = sorted;
        key.internal[0] = ctx->bStats.p; key.internal[1] = ctx->bMin.p; key.internal[2] = ctx->bHead.p;
        key.internal[3] = ctx->bOrder.p; key.internal[4] = ctx->bBin.p; key.internal[5] = ctx->gws.p;
        key.internal[6] = ctx->hStats;
        key.internal[7] = ctx->bAtt.p;
        key.attValid = io.attemptsValid;
        key.mech = ctx->M.rx;
        if (!ctx->gexec || std::memcmp(&key, &ctx->gkey, sizeof(key)) != 0) {
            if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
            ctx->gexec = nullptr;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = enqueue_prologue();
            WorkQueue q{ctx->bHead.p + QC_HEAD, ctx->bOrder.p, 0, ctx->bHead.p + QC_LEN};
            if (e == cudaSuccess)
                e = launch_integrate(sh.lc, sh.mixed, ctx->M, ko, sh.L, io, q, sh.global ? ctx->gws.p : nullptr, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(hs, ctx->bStats.p, ST_COUNT * sizeof(long long), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(hmin, ctx->bMin.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
            cudaGraph_t gr = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(st, &gr);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->gexec, gr, 0);
            if (gr) cudaGraphDestroy(gr);
            if (e != cudaSuccess) {
                ctx->gexec = nullptr;
                cudaGetLastError();
                return cuda_err(ctx, e, "step graph capture");
            }
            std::memcpy(&ctx->gkey, &key, sizeof(key));
        }
        // the graph is timed as a whole (kernel_ms = the step)
        CK(cudaEventRecord(ctx->ev0, st));
        CK(cudaGraphLaunch(ctx->gexec, st));
        CK(cudaEventRecord(ctx->ev1, st));
    } else {
        CK(enqueue_prologue());
        int nActive = 0;
        CK(cudaMemcpyAsync(&nActive, ctx->bHead.p + QC_LEN, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        group = ctx->opt.mapping ? ctx->opt.mapping
                                 : lane_auto(ctx, nActive) ? (int)FCS_MAPPING_LANE : tuned_group(ctx, io, nActive);
        Shape sh;
        if (!make_shape(ctx, group, true, sh))
            return set_err(ctx, FCS_ERR_UNSUPPORTED, "no launch shape for this mapping");
        fcs_status s = ensure_gws(ctx, sh);
        if (s != FCS_OK) return s;
        WorkQueue q{ctx->bHead.p + QC_HEAD, ctx->bOrder.p, nActive};
        CK(cudaEventRecord(ctx->ev0, st));
        if (nActive > 0)
            CK(launch_integrate(sh.lc, sh.mixed, ctx->M, ko, sh.L, io, q, sh.global ? ctx->gws.p : nullptr, st));
        CK(cudaEventRecord(ctx->ev1, st));
        hs = hsLocal;
        CK(cudaMemcpyAsync(hs, ctx->bStats.p, ST_COUNT * sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hmin, ctx->bMin.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    }
    ctx->attN = nc;  // this call's kernels record the attempts of its cells
    if (!dev) {
        CK(cudaMemcpyAsync(T, io.T, nc * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Y, io.Y, (size_t)ns * nc * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(sub, io.subDt, nc * 8, cudaMemcpyDeviceToHost, st));
        if (RR) CK(cudaMemcpyAsync(RR, io.RR, (size_t)ns * nc * 8, cudaMemcpyDeviceToHost, st));
        if (status) CK(cudaMemcpyAsync(status, io.status, nc * 4, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaEventRecord(ctx->evc1, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0, cms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    cudaEventElapsedTime(&cms, ctx->evc0, ctx->evc1);
    cudaGetLastError();  // an elapsed-time query that failed must not leak into the caller's next check
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
    if (dtMin) {
        double m = 1e15;  // great
        if (hs[ST_CELLS] > 0) std::memcpy(&m, hmin, sizeof(m));
        const double dref = dtc ? 0 : dt;
        *dtMin = dtc ? m : std::min(m, 2 * dref);
    }
    if (hs[ST_FAILED] > 0) return set_err(ctx, FCS_ERR_CELLS, "some cells failed; see cell_status");
    return FCS_OK;
}

extern "C" fcs_status fcs_integrate(fcs_ctx* ctx, int64_t n, double dt, const double* p, const double* rho0,
                                    double* T, double* Y, double* sub, double* RR, int32_t* status,
                                    fcs_step_stats* stats, double* dtMin, int32_t flags) {
    return integrate_impl(ctx, n, dt, nullptr, p, rho0, T, Y, sub, RR, status, stats, dtMin, flags);
}

extern "C" fcs_status fcs_integrate_lts(fcs_ctx* ctx, int64_t n, const double* dt, const double* p,
                                        const double* rho0, double* T, double* Y, double* sub, double* RR,
                                        int32_t* status, fcs_step_stats* stats, double* dtMin, int32_t flags) {
    if (!dt) return set_err(ctx, FCS_ERR_INVALID, "delta_t array is null");
    return integrate_impl(ctx, n, 0.0, dt, p, rho0, T, Y, sub, RR, status, stats, dtMin, flags);
}

// ------------------------------------------------------------------------
// per-cell evaluations

static fcs_status eval_impl(fcs_ctx* ctx, int64_t nc, const double* p, const double* T, const double* rho,
                            const double* Y, double* out, double* J, double* Qdot, int mode, int32_t flags) {
    if (!ctx) return FCS_ERR_INVALID;
    if (!ctx->loaded) return set_err(ctx, FCS_ERR_STATE, "no mechanism loaded");
    if (fcs_status s = refuse_if_async_pending(ctx)) return s;
    if (nc < 0 || nc > (int64_t)INT32_MAX) return set_err(ctx, FCS_ERR_INVALID, "n_cells out of range");
    if (!p || !T || !Y || !out) return set_err(ctx, FCS_ERR_INVALID, "null array");
    if (nc == 0) return FCS_OK;
    cudaSetDevice(ctx->device);
    const int ns = ctx->M.ns, n = ctx->M.n;
    const bool dev = flags & FCS_PTR_DEVICE;
    cudaStream_t st = ctx->stream;
    const size_t nout = (size_t)(mode == 3 ? 1 : mode == 2 ? ns : n) * nc;
    if ((mode == 2 || mode == 3) && !rho) return set_err(ctx, FCS_ERR_INVALID, "null rho");
    const double *dp = p, *dT = T, *dY = Y, *drho = rho;
    double *dout = out, *dJ = J, *dQ = Qdot;
    if (!dev) {
        CK(ctx->bp.ensure(nc)); CK(ctx->bT.ensure(nc)); CK(ctx->bY.ensure((size_t)ns * nc));
        CK(ctx->bOut.ensure(nout));
        CK(cudaMemcpyAsync(ctx->bp.p, p, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bT.p, T, nc * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bY.p, Y, (size_t)ns * nc * 8, cudaMemcpyHostToDevice, st));
        dp = ctx->bp.p; dT = ctx->bT.p; dY = ctx->bY.p; dout = ctx->bOut.p;
        if (mode == 2 || mode == 3) {
            CK(ctx->brho.ensure(nc));
            CK(cudaMemcpyAsync(ctx->brho.p, rho, nc * 8, cudaMemcpyHostToDevice, st));
            drho = ctx->brho.p;
        }
        if (J) { CK(ctx->bJ.ensure((size_t)n * n * nc)); dJ = ctx->bJ.p; }
        if (Qdot) { CK(ctx->bQ.ensure(nc)); dQ = ctx->bQ.p; }
    }
    // the per-cell evaluations run on cell groups (the lane mapping is the integrator's)
    const int group = ctx->opt.mapping > FCS_MAPPING_LANE ? ctx->opt.mapping : default_group(ctx);
    Shape sh;
    if (!make_shape(ctx, group, false, sh)) return set_err(ctx, FCS_ERR_UNSUPPORTED, "no launch shape");
    const int gpb = sh.lc.block / sh.lc.group;
    sh.lc.grid = (int)((nc + gpb - 1) / gpb);
    char* gws = nullptr;
    if (sh.global) {
        if (ctx->gws.ensure((size_t)sh.lc.grid * gpb * sh.L.bytes) != cudaSuccess)
            return set_err(ctx, FCS_ERR_NOMEM, "workspace allocation failed");
        gws = ctx->gws.p;
    }
    const KOpts ko = kopts(ctx->opt);
    CK(launch_eval(sh.lc, sh.mixed, ctx->M, ko, sh.L, nc, dp, dT, drho, dY, dout, dJ, dQ, mode, gws, st));
    if (!dev) {
        CK(cudaMemcpyAsync(out, dout, nout * 8, cudaMemcpyDeviceToHost, st));
        if (J) CK(cudaMemcpyAsync(J, dJ, (size_t)n * n * nc * 8, cudaMemcpyDeviceToHost, st));
        if (Qdot) CK(cudaMemcpyAsync(Qdot, dQ, nc * 8, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    return FCS_OK;
}

extern "C" fcs_status fcs_rhs(fcs_ctx* ctx, int64_t n, const double* p, const double* T, const double* Y,
                              double* dydt, int32_t flags) {
    return eval_impl(ctx, n, p, T, nullptr, Y, dydt, nullptr, nullptr, 0, flags);
}

extern "C" fcs_status fcs_jacobian(fcs_ctx* ctx, int64_t n, const double* p, const double* T, const double* Y,
                                   double* J, double* dydt, int32_t flags) {
    if (!J) return set_err(ctx, FCS_ERR_INVALID, "null J");
    return eval_impl(ctx, n, p, T, nullptr, Y, dydt, J, nullptr, 1, flags);
}

extern "C" fcs_status fcs_tc(fcs_ctx* ctx, int64_t n, const double* p, const double* T, const double* rho,
                             const double* Y, double* tc, int32_t flags) {
    return eval_impl(ctx, n, p, T, rho, Y, tc, nullptr, nullptr, 3, flags);
}

extern "C" fcs_status fcs_rates(fcs_ctx* ctx, int64_t n, const double* p, const double* T, const double* rho,
                                const double* Y, double* RR, double* Qdot, int32_t flags) {
    return eval_impl(ctx, n, p, T, rho, Y, RR, nullptr, Qdot, 2, flags);
}
