// fcs_ctx.h -- the context object behind the opaque fcs_ctx handle and the
// host-side helpers shared by the C ABI translation units (fcs_capi.cu,
// fcs_noalloc.cu).  Internal: not part of the public headers.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <string>
#include <tuple>

#include "../../include/fcs.h"
#include "fcs_device.cuh"
#include "fcs_internal.h"
#include "fcs_launch.h"

namespace fcs {

// Allocation failures injected by fcs_test_fail_allocations (host side: the
// next k growths of a device buffer report cudaErrorMemoryAllocation without
// calling cudaMalloc).
bool take_injected_alloc_failure();

template<class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t want) {
        if (want <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (take_injected_alloc_failure()) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(want, 1) * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// What a captured step graph depends on: the arrays, sizes and options.
struct GraphKey {
    const void *p, *rho0, *T, *Y, *sub, *RR, *status, *dtc;
    const void* internal[8];  // the context's buffers the graph uses (they move when they grow)
    const void* mech;         // the mechanism's device arrays (reloading replaces them)
    long long nc;
    double dt;
    fcs_options opt;
    int group;
    int sorted;
    int attValid;             // the queue is ordered by the previous call's per-cell attempts
};

struct GateState;             // surrogate gate (fcs_gate.cu)
void gate_release(fcs_ctx* ctx);

struct Shape {
    LaunchCfg lc;
    SlotLayout L;
    bool global;      // workspace in global memory
    bool mixed;
};

}  // namespace fcs

struct fcs_ctx {
    int device = 0;
    int numSMs = 0;
    size_t maxSmemPerBlock = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evc0 = nullptr, evc1 = nullptr;
    std::string err;
    // mechanism
    bool loaded = false;
    fcs::DevMech M{};
    fcs::DBuf<double> dW, dInvW, dTc, dCoef, dEff, dPlogRow, dPlogTa, dHf, dFo;
    fcs::DBuf<fcs::RxnInfo> dRx;
    fcs::DBuf<int> dPlogOff, dIncOff, dInc, dTbInc;
    // options
    fcs_options opt{};
    // per-call buffers
    fcs::DBuf<double> bp, brho, bT, bY, bSub, bRR, bDt, bOut, bJ, bQ;
    fcs::DBuf<int> bStatus, bOrder, bHead;
    fcs::DBuf<long long> bStats;
    fcs::DBuf<unsigned long long> bMin;
    fcs::DBuf<char> gws;
    std::map<std::tuple<int, int, int, int>, int> tuned;  // (n, precision, solver, jac) -> group
    fcs::GateState* gate = nullptr;                       // attached surrogate, if any
    // per-cell attempts of the last integration, for the cost-ordered queue
    fcs::DBuf<int> bAtt;
    long long attN = 0;                                   // batch size bAtt describes (0: none)
    // CUDA-graph step (FCS_CUDA_GRAPH)
    fcs::DBuf<int> bBin;                                  // predicted-step bin per cell
    cudaGraphExec_t gexec = nullptr;
    fcs::GraphKey gkey{};
    long long* hStats = nullptr;                          // pinned: ST_COUNT counters + min sub-step bits
    // asynchronous step (fcs_integrate_async / fcs_sync)
    cudaEvent_t evAsync = nullptr;
    bool asyncPending = false;
    double asyncDt = 0;
    int asyncGroup = 0;
};

namespace fcs {

fcs_status set_err(fcs_ctx* c, fcs_status s, const std::string& m);
// FCS_ERR_NOMEM for a failed allocation, FCS_ERR_CUDA otherwise
fcs_status cuda_err(fcs_ctx* c, cudaError_t e, const char* where);
// FCS_ERR_STATE while an fcs_integrate_async step is in flight on this
// context: its kernels read the context's queue, counters, workspace and
// mechanism, and fcs_sync reads its events and pinned statistics.
fcs_status refuse_if_async_pending(fcs_ctx* ctx);
// A cell array handed over as device memory must be device (or managed)
// memory of the context's device, aligned to `align` bytes: host memory
// handed to a kernel would fault.
fcs_status check_device_array(fcs_ctx* ctx, const void* ptr, const char* name, size_t align);
KOpts kopts(const fcs_options& o);
// Launch shape for a group size; false when impossible.
bool make_shape(fcs_ctx* ctx, int group, bool integrate, Shape& sh);
int default_group(fcs_ctx* ctx);
// The option's mapping, else one the autotuner cached for this key, else the default.
int cached_group(fcs_ctx* ctx);
// AUTO mapping: the lane mapping for this many reacting cells?
bool lane_auto(fcs_ctx* ctx, long long cells);
// Global-memory workspace for shapes whose slot exceeds shared memory.
fcs_status ensure_gws(fcs_ctx* ctx, const Shape& sh);

}  // namespace fcs

#define CK(call)                                                       \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return fcs::cuda_err(ctx, e_, #call);   \
    } while (0)
