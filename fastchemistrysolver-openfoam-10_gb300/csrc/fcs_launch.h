// fcs_launch.h -- kernel launch interface between the C ABI layer and the
// sm_103a kernels.
#pragma once
#include <cuda_runtime.h>
#include "fcs_internal.h"

namespace fcs {

struct SlotLayout;

// Device views of the per-call cell fields (species-major Y).
struct CellIO {
    long long nCells;
    double deltaT;
    const double* dtPerCell;   // LTS variant, or null
    const double* p;
    const double* rho0;
    double* T;
    double* Y;
    double* subDt;
    double* RR;                // may be null
    int* status;               // may be null
    long long* stats;          // ST_COUNT counters
    unsigned long long* dtMinBits;  // min of the uncapped sub-steps (positive-double bits)
    int* attempts;             // per cell: attempted steps of its last integration (written; may be null)
    int attemptsValid;         // attempts[] holds this batch's counts from the previous call: the
                               // binned queue orders the cells by it (most attempts first)
};

struct WorkQueue {
    int* head;                 // next queue index (atomic)
    const int* order;          // queue position -> cell, or null for identity
    int n;                     // queue length
    const int* nDev;           // if set, the queue length is read from device memory instead
};

// Work-queue counters (int) of the binned queue: next position, length,
// cells per bin, cells placed per bin, and a spare counter for callers.
constexpr int kQueueBins = 64;
enum { QC_HEAD = 0, QC_LEN = 1, QC_BINS = 2, QC_FILL = QC_BINS + kQueueBins, QC_AUX = QC_FILL + kQueueBins,
       QC_COUNT };

#ifdef __CUDACC__
// Queue bin of a cell whose previous integration took `attempts` attempted
// steps: eight bins per octave from 8 to 2048 attempts (0: cheapest).
__device__ __forceinline__ int attempt_bin(int attempts) {
    const int b = (int)floorf(8.f * log2f((float)(attempts > 1 ? attempts : 1))) - 24;
    return b < 0 ? 0 : (b >= kQueueBins ? kQueueBins - 1 : b);
}
#endif

struct LaunchCfg {
    int group;                 // threads per cell: 32, 64, 128, 256, or 1 (lane per cell)
    int block;                 // threads per block
    int grid;                  // blocks
};

cudaError_t launch_integrate(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                             const SlotLayout& L, const CellIO& io, const WorkQueue& q, char* gws,
                             cudaStream_t st);
cudaError_t launch_eval(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                        const SlotLayout& L, long long nc, const double* p, const double* T,
                        const double* rho, const double* Y, double* out, double* J, double* Qdot,
                        int mode, char* gws, cudaStream_t st);
cudaError_t launch_classify(const CellIO& io, int ns, double Treact, int* order, int* count,
                            cudaStream_t st);
cudaError_t integrate_attributes(int group, bool mixed, int* maxThreads, int* regs);
// Treact skip (as launch_classify) and, for the reacting cells, the bin of
// their predicted cost: the attempted steps of their previous integration
// when io.attemptsValid (bin = floor(8 log2(attempts)) - 24, eight bins per
// octave from 8 to 2048 attempts), else the step count delta_t / sub_delta_t
// (bin = floor(log2), 0..31); bin[c] = -1 for skipped cells.
cudaError_t launch_classify_binned(const CellIO& io, int ns, double Treact, int* bin, int* counters,
                                   cudaStream_t st);
// order[] = cells with bin >= 0, highest bin first; counters[QC_LEN] = their count.
cudaError_t launch_queue(long long nc, const int* bin, int* counters, int* order, cudaStream_t st);

// The lane-per-cell integrator (fcs_lane.cu): lc.group == 1, lc.block
// threads per block, one cell per thread; gws holds make_lane_layout(...).words
// doubles per thread of the grid.
cudaError_t launch_lane_integrate(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                                  const CellIO& io, const WorkQueue& q, char* gws, cudaStream_t st);
cudaError_t lane_attributes(bool mixed, int* maxThreads, int* regs);

// per-group-size instantiations (fcs_kernels_g<G>.cu)
template<int G>
cudaError_t launch_integrate_g(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                               const SlotLayout& L, const CellIO& io, const WorkQueue& q, char* gws,
                               cudaStream_t st);
template<int G>
cudaError_t launch_eval_g(const LaunchCfg& lc, bool mixed, const DevMech& M, const KOpts& o,
                          const SlotLayout& L, long long nc, const double* p, const double* T,
                          const double* rho, const double* Y, double* out, double* J, double* Qdot,
                          int mode, char* gws, cudaStream_t st);
template<int G>
cudaError_t integrate_attributes_g(bool mixed, int* maxThreads, int* regs);

}  // namespace fcs
