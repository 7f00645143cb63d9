// Instantiations of the cell-group kernels for groups of 256 threads (one
// translation unit per group size so that the build compiles them in parallel).
#include "fcs_kernels.cuh"

namespace fcs {

template<>
cudaError_t launch_integrate_g<256>(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                                  const SlotLayout& L, const CellIO& io, const WorkQueue& q, char* gws,
                                  cudaStream_t st) {
    return mixed ? launch_integrate_t<256, float>(lc, M, o, L, io, q, gws, st)
                 : launch_integrate_t<256, double>(lc, M, o, L, io, q, gws, st);
}

template<>
cudaError_t launch_eval_g<256>(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                             const SlotLayout& L, long long nc, const double* p, const double* T,
                             const double* rho, const double* Y, double* out, double* J, double* Qdot,
                             int mode, char* gws, cudaStream_t st) {
    return mixed ? launch_eval_t<256, float>(lc, M, o, L, nc, p, T, rho, Y, out, J, Qdot, mode, gws, st)
                 : launch_eval_t<256, double>(lc, M, o, L, nc, p, T, rho, Y, out, J, Qdot, mode, gws, st);
}

template<>
cudaError_t integrate_attributes_g<256>(bool mixed, int* maxThreads, int* regs) {
    return mixed ? attrs_t<256, float>(maxThreads, regs) : attrs_t<256, double>(maxThreads, regs);
}

}  // namespace fcs
