// fcs_async.cu -- fcs_integrate_async / fcs_sync: the batched integrate over
// caller-owned device arrays enqueued on the caller's CUDA stream, without a
// host round trip, so that a flow solver can overlap chemistry with its own
// work on other streams.  The step is the same device work as
// fcs_integrate's (classify with predicted-step bins, ordered queue,
// persistent integrator reading the queue length on the device); the
// counters and the minimum sub-step land in pinned host memory and are read
// by fcs_sync.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <string>
#include <thread>

#include "../../include/fcs.h"
#include "fcs_ctx.h"

using namespace fcs;

extern "C" fcs_status fcs_integrate_async(fcs_ctx* ctx, int64_t nc, double dt, const double* p, const double* rho0,
                                          double* T, double* Y, double* sub, double* RR, int32_t* status,
                                          int32_t flags, void* cuda_stream) {
    if (!ctx) return FCS_ERR_INVALID;
    if (!ctx->loaded) return set_err(ctx, FCS_ERR_STATE, "no mechanism loaded");
    if (ctx->asyncPending) return set_err(ctx, FCS_ERR_STATE, "a step is already in flight: call fcs_sync first");
    if (nc < 0 || nc > (int64_t)INT32_MAX) return set_err(ctx, FCS_ERR_INVALID, "n_cells out of range");
    if (!p || !rho0 || !T || !Y || !sub) return set_err(ctx, FCS_ERR_INVALID, "null cell array");
    if (!(dt > 0)) return set_err(ctx, FCS_ERR_INVALID, "delta_t must be positive");
    CK(cudaSetDevice(ctx->device));
    // the arrays must be device memory of this device: host memory would fault in the kernels
    {
        const struct { const void* ptr; const char* name; size_t align; } arrays[] = {
            {p, "p", 8}, {rho0, "rho0", 8}, {T, "T", 8}, {Y, "Y", 8}, {sub, "sub_delta_t", 8},
            {RR, "RR", 8}, {status, "cell_status", 4}};
        for (const auto& a : arrays)
            if (a.ptr)
                if (fcs_status s = check_device_array(ctx, a.ptr, a.name, a.align)) return s;
    }
    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : ctx->stream;
    const int ns = ctx->M.ns;
    const bool sorted = !(flags & FCS_NO_QUEUE_SORT);
    CK(ctx->bStats.ensure(ST_COUNT));
    CK(ctx->bMin.ensure(1));
    CK(ctx->bOrder.ensure(std::max<int64_t>(nc, 1)));
    CK(ctx->bHead.ensure(QC_COUNT));
    if (sorted) CK(ctx->bBin.ensure(std::max<int64_t>(nc, 1)));
    if (!ctx->hStats) CK(cudaMallocHost(&ctx->hStats, (ST_COUNT + 1) * sizeof(long long)));
    if (!ctx->evAsync) CK(cudaEventCreateWithFlags(&ctx->evAsync, cudaEventDisableTiming));
    const int group = lane_auto(ctx, nc) ? (int)FCS_MAPPING_LANE : cached_group(ctx);
    Shape sh;
    if (!make_shape(ctx, group, true, sh)) return set_err(ctx, FCS_ERR_UNSUPPORTED, "no launch shape for this mapping");
    fcs_status s = ensure_gws(ctx, sh);
    if (s != FCS_OK) return s;

    CellIO io{};
    io.nCells = nc;
    io.deltaT = dt;
    io.p = p; io.rho0 = rho0; io.T = T; io.Y = Y; io.subDt = sub; io.RR = RR; io.status = status;
    io.stats = ctx->bStats.p;
    io.dtMinBits = ctx->bMin.p;
    if (ctx->bAtt.n < (size_t)std::max<int64_t>(nc, 1)) ctx->attN = 0;
    CK(ctx->bAtt.ensure(std::max<int64_t>(nc, 1)));
    io.attempts = ctx->bAtt.p;
    io.attemptsValid = (sorted && ctx->attN == nc) ? 1 : 0;
    CK(cudaEventRecord(ctx->evc0, st));
    CK(cudaMemsetAsync(ctx->bStats.p, 0, ST_COUNT * sizeof(long long), st));
    CK(cudaMemsetAsync(ctx->bMin.p, 0x7f, sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(ctx->bHead.p, 0, QC_COUNT * sizeof(int), st));
    if (sorted) {
        CK(launch_classify_binned(io, ns, ctx->opt.T_react, ctx->bBin.p, ctx->bHead.p, st));
        CK(launch_queue(nc, ctx->bBin.p, ctx->bHead.p, ctx->bOrder.p, st));
    } else {
        CK(launch_classify(io, ns, ctx->opt.T_react, ctx->bOrder.p, ctx->bHead.p + QC_LEN, st));
    }
    WorkQueue q{ctx->bHead.p + QC_HEAD, ctx->bOrder.p, 0, ctx->bHead.p + QC_LEN};
    CK(cudaEventRecord(ctx->ev0, st));
    CK(launch_integrate(sh.lc, sh.mixed, ctx->M, kopts(ctx->opt), sh.L, io, q, sh.global ? ctx->gws.p : nullptr, st));
    CK(cudaEventRecord(ctx->ev1, st));
    CK(cudaMemcpyAsync(ctx->hStats, ctx->bStats.p, ST_COUNT * sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ctx->hStats + ST_COUNT, ctx->bMin.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ctx->evc1, st));
    CK(cudaEventRecord(ctx->evAsync, st));
    ctx->asyncPending = true;
    ctx->attN = nc;
    ctx->asyncDt = dt;
    ctx->asyncGroup = group;
    return FCS_OK;
}

static fcs_status sync_impl(fcs_ctx* ctx, double timeout_ms, fcs_step_stats* stats, double* dtMin) {
    if (!ctx) return FCS_ERR_INVALID;
    if (!ctx->asyncPending) return set_err(ctx, FCS_ERR_STATE, "no step in flight");
    CK(cudaSetDevice(ctx->device));
    if (timeout_ms >= 0) {
        // bounded host-side wait: poll the step's event until it completes or
        // the limit runs out; the step itself is left running and stays
        // pending, so a later fcs_sync / fcs_sync_timeout collects it
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const cudaError_t q = cudaEventQuery(ctx->evAsync);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return cuda_err(ctx, q, "cudaEventQuery(step)");
            const double el =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (el >= timeout_ms)
                return set_err(ctx, FCS_ERR_TIMEOUT, "the step did not complete within the wait limit");
            std::this_thread::sleep_for(std::chrono::microseconds(el < 1.0 ? 20 : 200));
        }
    }
    ctx->asyncPending = false;
    CK(cudaEventSynchronize(ctx->evAsync));
    const long long* hs = ctx->hStats;
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
        stats->mapping = ctx->asyncGroup;
        stats->reserved = 0;
    }
    if (dtMin) {
        double m = 1e15;
        if (hs[ST_CELLS] > 0) std::memcpy(&m, hs + ST_COUNT, sizeof(m));
        *dtMin = std::min(m, 2 * ctx->asyncDt);
    }
    if (hs[ST_FAILED] > 0) return set_err(ctx, FCS_ERR_CELLS, "some cells failed; see cell_status");
    return FCS_OK;
}

extern "C" fcs_status fcs_sync(fcs_ctx* ctx, fcs_step_stats* stats, double* dtMin) {
    return sync_impl(ctx, -1.0, stats, dtMin);
}

extern "C" fcs_status fcs_sync_timeout(fcs_ctx* ctx, double timeout_ms, fcs_step_stats* stats, double* dtMin) {
    if (!(timeout_ms >= 0)) return set_err(ctx, FCS_ERR_INVALID, "timeout_ms must be >= 0");
    return sync_impl(ctx, timeout_ms, stats, dtMin);
}
