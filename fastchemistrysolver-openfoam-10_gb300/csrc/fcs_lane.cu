// Launch code of the lane-per-cell integrator (fcs_lane.cuh).
#include "fcs_lane.cuh"

namespace fcs {

cudaError_t launch_lane_integrate(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                                  const CellIO& io, const WorkQueue& q, char* gws, cudaStream_t st) {
    if (!gws || lc.block % 32 != 0) return cudaErrorInvalidValue;
    const LaneLayout L = make_lane_layout(M.ns, M.nr, M.nTB, mixed);
    auto k = mixed ? lane_integrate_kernel<float> : lane_integrate_kernel<double>;
    // the workspace lives in global memory: all of the unified L1/shared
    // memory as L1, which caches the lanes' vectors and species arrays
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxL1);
    if (e != cudaSuccess) return e;
    k<<<lc.grid, lc.block, 0, st>>>(M, o, L, io, q, reinterpret_cast<double*>(gws));
    return cudaGetLastError();
}

cudaError_t lane_attributes(bool mixed, int* maxThreads, int* regs) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, mixed ? lane_integrate_kernel<float> : lane_integrate_kernel<double>);
    if (e != cudaSuccess) return e;
    *maxThreads = a.maxThreadsPerBlock;
    *regs = a.numRegs;
    return cudaSuccess;
}

}  // namespace fcs
