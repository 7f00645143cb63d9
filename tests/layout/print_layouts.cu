// Prints the per-cell workspace layouts the integrators use (host code only:
// no CUDA call, runs without a GPU), for tests/test_layouts.py to check that
// no two regions overlap and that each holds what the kernels put there.
#include <cstdio>

#include "fcs_device.cuh"
#include "fcs_lane_layout.h"

int main() {
    const int species[] = {1, 2, 9, 10, 13, 14, 15, 16, 23, 52, 53, 54, 110, 111, 139, 140, 199, 200, 254, 255};
    const int reactions[] = {0, 1, 27, 325, 784, 1500};
    const int thirdBody[] = {0, 3, 40};
    for (int ns : species)
        for (int nr : reactions)
            for (int ntb : thirdBody)
                for (int mixed = 0; mixed < 2; mixed++) {
                    const fcs::LaneLayout W = fcs::make_lane_layout(ns, nr, ntb, mixed);
                    std::printf("lane %d %d %d %d  %d %d %d %d %d %d %d %d %d %d %d\n", ns, nr, ntb, mixed, W.offA,
                                W.offVec, W.offSp, W.offTb, W.offInvD, W.offPiv, W.offLU32, W.offScale, W.offX32,
                                W.offRx, W.words);
                    for (int seulex = 0; seulex < 2; seulex++) {
                        const int chunks[] = {0, 1, 32, 128, nr, nr + 5};
                        for (int rc : chunks) {
                            const fcs::SlotLayout L = fcs::make_layout(ns, nr, ntb, mixed, seulex, rc);
                            std::printf("slot %d %d %d %d %d %d  %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d\n",
                                        ns, nr, ntb, mixed, seulex, rc, L.ld, L.offJ64, L.offLU64, L.offJ32,
                                        L.offLU32, L.offVec, L.offVec32, L.offSp, L.offInvD, L.offScale, L.offPiv,
                                        L.offRx, L.rc, L.offCur, L.offTb, L.offTable, L.offRed, L.bytes);
                        }
                    }
                }
    return 0;
}
