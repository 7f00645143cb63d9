// fcs_lane_layout.h -- per-lane workspace of the lane-per-cell integrator
// (fcs_lane.cuh), shared by the host launch code and the kernels.
//
// In the lane mapping one thread integrates one cell.  Its working set (the
// N x N iteration matrix, the stage vectors, the species scratch) lives in a
// global-memory workspace, interleaved across the 32 lanes of a warp: element
// e of a lane's array sits at warp_base[e * 32 + lane], so the 32 lanes of a
// warp, which run the same instruction on the same element index of their own
// cells, touch 256 contiguous bytes.  Offsets below are in doubles per lane.
#pragma once

namespace fcs {

constexpr int kLaneVecs = 13;  // stage / work vectors per lane (see fcs_lane.cuh)

struct LaneLayout {
    int n, ns, nr, nTB;
    int offA;     // [n*n] FP64 Jacobian / iteration matrix (row-major), LU factors in place (FP64 method)
    int offVec;   // kLaneVecs vectors of n doubles
    int offSp;    // 6 species arrays [ns]: C, B = exp(-G/RT), Binv, Cp, Ha, dB/dT
    int offTb;    // third-body concentration M and Jacobian weight [nTB] each
    int offInvD;  // [n] reciprocal pivots
    int offPiv;   // [n] int32 pivot rows (n/2 rounded up doubles)
    int offLU32;  // mixed precision: [n*n] FP32 LU factors (n*n/2 rounded up doubles)
    int offScale; // mixed precision: [2n] row and column equilibration factors
    int offX32;   // mixed precision: 2 vectors of n floats (n rounded up doubles)
    int offRx;    // [2 nr] per-reaction net rate q and its temperature derivative dq/dT
    int words;    // doubles per lane
};

inline LaneLayout make_lane_layout(int ns, int nr, int nTB, bool mixed) {
    LaneLayout L;
    const int n = ns + 1;
    L.n = n;
    L.ns = ns;
    L.nr = nr;
    L.nTB = nTB;
    int o = 0;
    L.offA = o;     o += n * n;
    L.offVec = o;   o += kLaneVecs * n;
    L.offSp = o;    o += 6 * ns;
    L.offTb = o;    o += 2 * (nTB > 0 ? nTB : 1);
    L.offInvD = o;  o += n;
    L.offPiv = o;   o += (n + 1) / 2;
    L.offLU32 = o;  if (mixed) o += (n * n + 1) / 2;
    L.offScale = o; if (mixed) o += 2 * n;
    L.offX32 = o;   if (mixed) o += n;
    L.offRx = o;    o += 2 * (nr > 0 ? nr : 1);
    L.words = o;
    return L;
}

}  // namespace fcs
