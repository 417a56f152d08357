"""Launch geometry of the warp-group kernel, checked on the host (no GPU):
ring depth, shared memory, warp counts, column groups and chunked ring slots
for every arithmetic and element size the kernel takes (afm_debug_segment_geometry)."""
import ctypes as C

import pytest

from amat_gb300 import _native

KINDS = {0: "fp64", 1: "split", 2: "fp32 hi plane", 3: "fp32 symmetric", 4: "corrected, fp32 u",
         5: "corrected, double-float u", 6: "corrected, fp32 rows"}
EIGHT_BYTE_U = {0, 1, 5}       # staged u of 8 bytes: up to 16 consumer warps
SMEM_LIMIT = 227 * 1024        # dynamic shared memory of one CTA
MAX_CHUNK = 8


def geometry(kind, n):
    out = (C.c_uint32 * 8)()
    assert _native.libafm().afm_debug_segment_geometry(kind, n, out) == 0
    chunk, stages, warps, groups, gc, smem, unit, copy = list(out)
    return dict(chunk=chunk, stages=stages, warps=warps, groups=groups, gc=gc, smem=smem, unit=unit, copy=copy)


@pytest.mark.parametrize("kind", sorted(KINDS))
@pytest.mark.parametrize("n", [17, 20, 24, 30, 32, 33, 48, 60, 64, 65, 96])
def test_ring_and_groups(kind, n):
    g = geometry(kind, n)
    gr = (n + 31) // 32
    assert g["gc"] == (2 if gr == 2 and kind in EIGHT_BYTE_U else 1)
    assert g["warps"] == g["groups"] * gr * g["gc"]
    assert g["warps"] <= (16 if kind in EIGHT_BYTE_U else 24)
    # every group holds one slot while a further two are in flight
    assert g["stages"] >= g["groups"] + 2 or (g["groups"] == 1 and g["stages"] >= 2)
    assert g["smem"] <= SMEM_LIMIT
    assert 1 <= g["chunk"] <= MAX_CHUNK
    if g["copy"] < g["unit"]:  # hi plane only: units are not contiguous in the copied part
        assert g["chunk"] == 1
    assert g["chunk"] * g["copy"] <= 16384 or g["chunk"] == 1


def test_known_layouts():
    # hex20 (n = 60) split: single units of 28.8 KB, four warps per element, four elements per SM
    h20 = geometry(1, 60)
    assert (h20["chunk"], h20["gc"], h20["groups"]) == (1, 2, 4)
    assert h20["unit"] == 28800
    # hex8 elasticity (n = 24): two split units per slot, six symmetric FP32 units per slot
    assert geometry(1, 24)["chunk"] == 2
    assert geometry(3, 24)["chunk"] == 6
    # one-warp groups keep every consumer warp (no named-barrier limit of 15 groups)
    assert geometry(3, 24)["groups"] == 24


def test_bad_arguments():
    out = (C.c_uint32 * 8)()
    lib = _native.libafm()
    for kind, n in [(-1, 24), (7, 24), (1, 16), (1, 97)]:
        assert lib.afm_debug_segment_geometry(kind, n, out) == 105  # AFM_ERR_INVALID_ARG
