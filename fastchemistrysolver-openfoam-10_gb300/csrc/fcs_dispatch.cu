// fcs_dispatch.cu -- run-time dispatch over the per-group-size kernel
// instantiations, and the cell classification kernel.
#include "fcs_kernels.cuh"

namespace fcs {

// Treact skip + compaction of the active cells into the work queue
__global__ void classify_kernel(CellIO io, int ns, double Treact, int* order, int* count) {
    const long long nc = io.nCells;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nc;
         c += (long long)gridDim.x * blockDim.x) {
        if (io.T[c] > Treact) {
            const int k = atomicAdd(count, 1);
            order[k] = (int)c;
        } else {
            if (io.RR) for (int i = 0; i < ns; i++) io.RR[(size_t)i * nc + c] = 0;
            if (io.status) io.status[c] = FCS_CELL_SKIPPED;
            atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_SKIPPED]), 1ull);
        }
    }
}

__device__ __forceinline__ int step_bin(double deltaT, double sub) {
    const double steps = deltaT / fmax(sub, 1e-300);
    int b = steps > 1 ? (int)log2(steps) : 0;
    return b < 0 ? 0 : (b >= 32 ? 31 : b);
}

__global__ void classify_bin_kernel(CellIO io, int ns, double Treact, int* bin, int* counters) {
    __shared__ int hist[kQueueBins];
    for (int b = threadIdx.x; b < kQueueBins; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    const long long nc = io.nCells;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nc;
         c += (long long)gridDim.x * blockDim.x) {
        if (io.T[c] > Treact) {
            const double deltaT = io.dtPerCell ? io.dtPerCell[c] : io.deltaT;
            const int b = io.attemptsValid ? attempt_bin(io.attempts[c]) : step_bin(deltaT, io.subDt[c]);
            bin[c] = b;
            atomicAdd(&hist[b], 1);
        } else {
            bin[c] = -1;
            if (io.RR) for (int i = 0; i < ns; i++) io.RR[(size_t)i * nc + c] = 0;
            if (io.status) io.status[c] = FCS_CELL_SKIPPED;
            atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_SKIPPED]), 1ull);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kQueueBins; b += blockDim.x)
        if (hist[b]) atomicAdd(&counters[QC_BINS + b], hist[b]);
}

__global__ void queue_kernel(long long nc, const int* __restrict__ bin, int* counters, int* __restrict__ order) {
    __shared__ int start[kQueueBins];
    if (threadIdx.x == 0) {
        int s = 0;
        for (int b = kQueueBins - 1; b >= 0; b--) {
            start[b] = s;
            s += counters[QC_BINS + b];
        }
        if (blockIdx.x == 0) counters[QC_LEN] = s;
    }
    __syncthreads();
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nc;
         c += (long long)gridDim.x * blockDim.x) {
        const int b = bin[c];
        if (b >= 0) order[start[b] + atomicAdd(&counters[QC_FILL + b], 1)] = (int)c;
    }
}

cudaError_t launch_classify_binned(const CellIO& io, int ns, double Treact, int* bin, int* counters,
                                   cudaStream_t st) {
    const int block = 256;
    long long blocks = (io.nCells + block - 1) / block;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    classify_bin_kernel<<<(int)blocks, block, 0, st>>>(io, ns, Treact, bin, counters);
    return cudaGetLastError();
}

cudaError_t launch_queue(long long nc, const int* bin, int* counters, int* order, cudaStream_t st) {
    const int block = 256;
    long long blocks = (nc + block - 1) / block;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    queue_kernel<<<(int)blocks, block, 0, st>>>(nc, bin, counters, order);
    return cudaGetLastError();
}

cudaError_t launch_integrate(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                             const SlotLayout& L, const CellIO& io, const WorkQueue& q, char* gws,
                             cudaStream_t st) {
    switch (lc.group) {
        case 1: return launch_lane_integrate(lc, mixed, M, o, io, q, gws, st);
        case 32: return launch_integrate_g<32>(lc, mixed, M, o, L, io, q, gws, st);
        case 64: return launch_integrate_g<64>(lc, mixed, M, o, L, io, q, gws, st);
        case 128: return launch_integrate_g<128>(lc, mixed, M, o, L, io, q, gws, st);
        case 256: return launch_integrate_g<256>(lc, mixed, M, o, L, io, q, gws, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_eval(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                        const SlotLayout& L, long long nc, const double* p, const double* T,
                        const double* rho, const double* Y, double* out, double* J, double* Qdot,
                        int mode, char* gws, cudaStream_t st) {
    switch (lc.group) {
        case 32: return launch_eval_g<32>(lc, mixed, M, o, L, nc, p, T, rho, Y, out, J, Qdot, mode, gws, st);
        case 64: return launch_eval_g<64>(lc, mixed, M, o, L, nc, p, T, rho, Y, out, J, Qdot, mode, gws, st);
        case 128: return launch_eval_g<128>(lc, mixed, M, o, L, nc, p, T, rho, Y, out, J, Qdot, mode, gws, st);
        case 256: return launch_eval_g<256>(lc, mixed, M, o, L, nc, p, T, rho, Y, out, J, Qdot, mode, gws, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t integrate_attributes(int group, bool mixed, int* maxThreads, int* regs) {
    switch (group) {
        case 1: return lane_attributes(mixed, maxThreads, regs);
        case 32: return integrate_attributes_g<32>(mixed, maxThreads, regs);
        case 64: return integrate_attributes_g<64>(mixed, maxThreads, regs);
        case 128: return integrate_attributes_g<128>(mixed, maxThreads, regs);
        case 256: return integrate_attributes_g<256>(mixed, maxThreads, regs);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_classify(const CellIO& io, int ns, double Treact, int* order, int* count,
                            cudaStream_t st) {
    const int block = 256;
    long long blocks = (io.nCells + block - 1) / block;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    classify_kernel<<<(int)blocks, block, 0, st>>>(io, ns, Treact, order, count);
    return cudaGetLastError();
}

}  // namespace fcs
