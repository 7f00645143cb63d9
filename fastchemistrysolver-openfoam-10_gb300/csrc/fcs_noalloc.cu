// fcs_noalloc.cu -- fcs_integrate_noalloc: the batched integrate entry point
// for callers that must not allocate device memory during a time step.
//
// Who needs it: a flow solver that hands all free device memory to its own
// pool at start-up (so a cudaMalloc inside the chemistry call would fail part
// way through a run), and one that keeps other streams busy while chemistry
// runs (cudaMalloc/cudaFree of the grow-only buffers behind fcs_integrate
// synchronise the device whenever the number of reacting cells grows).
//
// Everything the call needs beyond the caller's own device arrays and the
// mechanism (uploaded once by fcs_load_mechanism) lives in one file-scope
// device array, g_noalloc_scratch: the step counters, the minimum sub-step,
// the work-queue head and the queue of reacting cells, at most
// FCS_NOALLOC_MAX_CELLS of them.  The per-cell Rosenbrock/Seulex slot must
// fit in shared memory (there is no global-memory workspace here).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/fcs.h"
#include "fcs_ctx.h"

using namespace fcs;

namespace {

constexpr long long kMaxCells = FCS_NOALLOC_MAX_CELLS;
// Byte layout of the scratch:
//   [0, 128)    step counters, ST_COUNT long longs      -- zeroed every call
//   [128, 136)  minimum uncapped sub-step, double bits   -- set to 0x7f.. every call
//   [136, 144)  work-queue head, reacting-cell count     -- zeroed every call
//   [256, ...)  queue of reacting cells (int32 per cell) -- written by the classify pass
constexpr size_t kStatsOff = 0, kMinOff = 128, kHeadOff = 136, kOrderOff = 256;
constexpr size_t kScratchBytes = kOrderOff + sizeof(int) * (size_t)kMaxCells;
static_assert(ST_COUNT * sizeof(long long) <= kMinOff, "counter block too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_base[kMaxDevices] = {};

// Device address of this device's copy of the scratch.  The first call on a
// device (which must be the current device) looks it up with
// cudaGetSymbolAddress; that lookup may load this file's device module, so the
// first call should be made before any stream capture begins.
fcs_status scratch_base(fcs_ctx* ctx, unsigned char** out) {
    const int dev = ctx->device;
    if (dev < 0 || dev >= kMaxDevices) return set_err(ctx, FCS_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_base[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_base[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_base[dev];
    return FCS_OK;
}

}  // namespace

extern "C" fcs_status fcs_integrate_noalloc(fcs_ctx* ctx, int64_t nc, double dt, const double* p,
                                            const double* rho0, double* T, double* Y, double* sub,
                                            double* RR, int32_t* status, fcs_step_stats* stats,
                                            double* dtMin) {
    fcs_status s0;
    if (!ctx) return FCS_ERR_INVALID;
    if (!ctx->loaded) return set_err(ctx, FCS_ERR_STATE, "no mechanism loaded");
    // a pending asynchronous step still reads the context's events and stream
    if ((s0 = refuse_if_async_pending(ctx)) != FCS_OK) return s0;
    if (nc < 0 || nc > kMaxCells)
        return set_err(ctx, FCS_ERR_INVALID,
                       "n_cells out of range: fcs_integrate_noalloc takes at most " +
                           std::to_string(kMaxCells) + " cells per call (FCS_NOALLOC_MAX_CELLS)");
    if (!(dt > 0)) return set_err(ctx, FCS_ERR_INVALID, "delta_t must be positive");
    if (!p || !rho0 || !T || !Y || !sub) return set_err(ctx, FCS_ERR_INVALID, "null cell array");
    CK(cudaSetDevice(ctx->device));
    fcs_status s;
    const struct { const void* ptr; const char* name; size_t align; } arrays[] = {
        {p, "p", 8}, {rho0, "rho0", 8}, {T, "T", 8}, {Y, "Y", 8}, {sub, "sub_delta_t", 8},
        {RR, "RR", 8}, {status, "cell_status", 4}};
    for (const auto& a : arrays)
        if (a.ptr && (s = check_device_array(ctx, a.ptr, a.name, a.align)) != FCS_OK) return s;
    unsigned char* base = nullptr;
    if ((s = scratch_base(ctx, &base)) != FCS_OK) return s;

    const int ns = ctx->M.ns;
    cudaStream_t st = ctx->stream;
    long long* dStats = reinterpret_cast<long long*>(base + kStatsOff);
    unsigned long long* dMin = reinterpret_cast<unsigned long long*>(base + kMinOff);
    int* dHead = reinterpret_cast<int*>(base + kHeadOff);
    int* dOrder = reinterpret_cast<int*>(base + kOrderOff);

    CellIO io{};
    io.nCells = nc;
    io.deltaT = dt;
    io.dtPerCell = nullptr;
    io.p = p; io.rho0 = rho0; io.T = T; io.Y = Y; io.subDt = sub; io.RR = RR; io.status = status;
    io.stats = dStats;
    io.dtMinBits = dMin;

    CK(cudaEventRecord(ctx->evc0, st));
    CK(cudaMemsetAsync(base, 0, kOrderOff, st));
    CK(cudaMemsetAsync(dMin, 0x7f, sizeof(unsigned long long), st));
    // classify: cells with T <= Treact are skipped (transientSolve.H:39, 70-76)
    CK(launch_classify(io, ns, ctx->opt.T_react, dOrder, dHead + 1, st));
    int nActive = 0;
    CK(cudaMemcpyAsync(&nActive, dHead + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));

    // The autotuner allocates its trial copies, so it is not run here: an
    // explicit mapping, else one the autotuner cached for this key, else the
    // default for the mechanism size.
    int group = ctx->opt.mapping;
    if (!group) {
        const auto key = std::make_tuple(ctx->M.n, (int)ctx->opt.precision, (int)ctx->opt.solver, (int)ctx->opt.jacobian);
        const auto it = ctx->tuned.find(key);
        group = it != ctx->tuned.end() ? it->second : default_group(ctx);
    }
    Shape sh;
    if (!make_shape(ctx, group, true, sh))
        return set_err(ctx, FCS_ERR_UNSUPPORTED, "no launch shape for this mapping");
    if (sh.global)
        return set_err(ctx, FCS_ERR_UNSUPPORTED,
                       "per-cell workspace of " + std::to_string(sh.L.bytes) +
                           " bytes exceeds shared memory; fcs_integrate_noalloc has no global workspace");
    WorkQueue q{dHead, dOrder, nActive};
    const KOpts ko = kopts(ctx->opt);
    CK(cudaEventRecord(ctx->ev0, st));
    if (nActive > 0) CK(launch_integrate(sh.lc, sh.mixed, ctx->M, ko, sh.L, io, q, nullptr, st));
    CK(cudaEventRecord(ctx->ev1, st));
    long long hs[ST_COUNT];
    unsigned long long hmin = 0;
    CK(cudaMemcpyAsync(hs, dStats, sizeof(hs), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&hmin, dMin, sizeof(hmin), cudaMemcpyDeviceToHost, st));
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
        double m = 1e15;
        if (hs[ST_CELLS] > 0) std::memcpy(&m, &hmin, sizeof(m));
        *dtMin = std::min(m, 2 * dt);
    }
    if (hs[ST_FAILED] > 0) return set_err(ctx, FCS_ERR_CELLS, "some cells failed; see cell_status");
    return FCS_OK;
}
