"""The per-cell workspaces of the integrators, checked on the host: every
region the kernels write (fcs_device.cuh make_slot / make_layout for the
cell groups, fcs_lane_layout.h for the lane mapping) is as large as what
they put there and overlaps no other region, for mechanism sizes from 1 to
255 species.  A region too small would be an out-of-bounds write on the GPU;
the check runs here, without one."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "fastchemistrysolver-openfoam-10_gb300", "csrc")
KNV = 12          # stage vectors of a cell-group slot
KLANEVECS = 13    # stage vectors of a lane


@pytest.fixture(scope="module")
def layouts(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("layouts") / "print_layouts")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + CSRC, "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "layout", "print_layouts.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    lane = [list(map(int, ln.split()[1:])) for ln in out if ln.startswith("lane ")]
    slot = [list(map(int, ln.split()[1:])) for ln in out if ln.startswith("slot ")]
    assert lane and slot
    return lane, slot


def _disjoint(regions, what):
    live = sorted((a, a + n, name) for name, a, n in regions if n > 0)
    for (a0, e0, n0), (a1, e1, n1) in zip(live, live[1:]):
        assert e0 <= a1, f"{what}: {n0} [{a0}, {e0}) overlaps {n1} [{a1}, {e1})"
    return live[-1][1]


def test_lane_workspace_regions(layouts):
    lane, _ = layouts
    for ns, nr, ntb, mixed, offA, offVec, offSp, offTb, offInvD, offPiv, offLU32, offScale, offX32, offRx, words \
            in lane:
        n = ns + 1
        what = f"lane ns={ns} nr={nr} nTB={ntb} mixed={mixed}"
        regions = [("A", offA, n * n), ("vec", offVec, KLANEVECS * n), ("species", offSp, 6 * ns),
                   ("third body", offTb, 2 * max(ntb, 1)), ("invD", offInvD, n),
                   ("piv (int32)", offPiv, (n + 1) // 2), ("q, dq/dT", offRx, 2 * max(nr, 1))]
        if mixed:
            regions += [("LU32 (float)", offLU32, (n * n + 1) // 2), ("scale", offScale, 2 * n),
                        ("x32, r32 (float)", offX32, n)]
        end = _disjoint(regions, what)
        assert end <= words, what


def test_cell_group_slot_regions(layouts):
    _, slot = layouts
    for (ns, nr, ntb, mixed, seulex, rc_in, ld, offJ64, offLU64, offJ32, offLU32, offVec, offVec32, offSp,
         offInvD, offScale, offPiv, offRx, rc, offCur, offTb, offTable, offRed, nbytes) in slot:
        n = ns + 1
        what = f"slot ns={ns} nr={nr} nTB={ntb} mixed={mixed} seulex={seulex} rc={rc_in}"
        assert ld >= n and ld % 2 == 1, what
        assert rc >= 1 and (nr == 0 or rc <= nr), what
        m64, m32 = n * ld * 8, n * ld * 4
        if seulex:
            matrices = [("J64", offJ64, m64), ("LU64", offLU64, m64)]
            if mixed:  # the FP32 factors live inside the FP64 LU region
                assert offLU64 <= offLU32 and offLU32 + m32 <= offLU64 + m64, what
        elif mixed:
            # FP64 Jacobian kept beside the FP32 factors; the FP64 fallback
            # factors the Jacobian in place
            assert offLU64 == offJ64, what
            matrices = [("J64", offJ64, m64), ("LU32", offLU32, m32)]
        else:
            assert offLU64 == offJ64, what
            matrices = [("J64 / LU64", offJ64, m64)]
        regions = matrices + [
            ("vectors", offVec, KNV * n * 8), ("species", offSp, 7 * ns * 8), ("invD", offInvD, n * 8),
            ("piv", offPiv, n * 4),
            # one chunk of Kf, Kr, q, dq/dT; also the LU's permutation (n ints)
            ("reaction chunk", offRx, max(4 * rc * 8, n * 4)),
            ("incidence cursor", offCur, ns * 4), ("third body", offTb, 2 * max(ntb, 1) * 8),
            ("reduction", offRed, 48 * 8)]
        if mixed:
            regions += [("x32, r32", offVec32, 2 * n * 4), ("scale", offScale, 2 * n * 8)]
        if seulex:
            regions += [("extrapolation table", offTable, 12 * n * 8)]
        end = _disjoint(regions, what)
        assert end <= nbytes and nbytes % 16 == 0, what
        for name, off, _ in regions:
            assert off % 16 == 0, f"{what}: {name} at {off}"


def test_headline_slot_and_lane_sizes(layouts):
    """The sizes the launch shapes are built on (53 species, 325 reactions,
    13 third-body rows): a 37.8 KB cell-group slot with reaction chunks of
    128, and 4,693 doubles (37.5 KB) per lane."""
    lane, slot = layouts
    n, nr, ntb = 54, 325, 13
    (row,) = [s for s in slot if s[:6] == [53, 325, 3, 0, 0, 128]]
    assert 37000 <= row[-1] <= 38500
    (w,) = [ln for ln in lane if ln[:4] == [53, 325, 3, 0]]
    # the same layout with 13 third-body rows: 20 more doubles than with 3
    assert w[-1] + 2 * (ntb - 3) == n * n + 13 * n + 6 * 53 + 2 * ntb + n + (n + 1) // 2 + 2 * nr == 4693
