"""The work dealing of the FP64 filter sweeps (host only): the launch shape
the library computes, replayed with the kernel's segment walk
(ns_kernels.cu k_filter), produces every pass-2 position of every line
exactly once, with exactly one exact start (pass 1) and one end (pass 3)
per line, for large, ragged and tiny sizes."""
import ctypes as C

import pytest

from navierstokes_gb300 import _lib as L


def plan(nslib, nlines, n, nk, warm, nsm=152):
    seg, blocks = C.c_int64(), C.c_int()
    assert nslib.ns_filter_plan(nlines, n, nk, warm, nsm, C.byref(seg), C.byref(blocks)) == 0
    return seg.value, blocks.value


def walk(nlines, n, nk, seg, blocks):
    """The per-warp loop of k_filter: pieces (k, line, a, b)."""
    gpk = (nlines + 31) // 32
    len2 = n - 12
    total = gpk * nk * len2
    for wid in range(blocks * 4):
        s0 = wid * seg
        s1 = min(total, s0 + seg)
        sp = s0
        while sp < s1:
            g = sp // len2
            e = min(s1, (g + 1) * len2)
            k, g0 = g // gpk, (g % gpk) * 32
            for lane in range(32):
                if g0 + lane < nlines:
                    yield k, g0 + lane, 6 + sp - g * len2, 6 + e - g * len2
            sp = e


@pytest.mark.parametrize("nlines,n,nk,warm", [
    (2048, 4096, 4, 44), (4096, 2048, 4, 44), (201, 201, 5, 44), (100, 37, 5, 44),
    (33, 13, 4, 44), (1000, 1000, 4, -1), (64, 200, 4, 44), (17, 25, 1, 3), (512, 512, 4, 44)])
def test_every_position_once(nslib, nlines, n, nk, warm):
    seg, blocks = plan(nslib, nlines, n, nk, warm)
    assert seg >= 1 and blocks >= 1
    pieces = {}
    for k, line, a, b in walk(nlines, n, nk, seg, blocks):
        assert 6 <= a < b <= n - 6
        pieces.setdefault((k, line), []).append((a, b))
    assert len(pieces) == nlines * nk
    for iv in pieces.values():
        iv.sort()
        assert iv[0][0] == 6 and iv[-1][1] == n - 6
        assert all(iv[q][1] == iv[q + 1][0] for q in range(len(iv) - 1))


def test_large_grids_use_two_warps_per_subpartition(nslib):
    seg, blocks = plan(nslib, 2048, 4096, 4, 44)
    assert blocks * 4 == 2 * 4 * 152            # 2 warps per sub-partition
    seg, blocks = plan(nslib, 512, 512, 4, 44)
    assert blocks * 4 <= 4 * 152                # short segments: one warp each


def test_bad_arguments(nslib):
    seg, blocks = C.c_int64(), C.c_int()
    assert nslib.ns_filter_plan(0, 100, 4, 44, 152, C.byref(seg), C.byref(blocks)) == L.NS_ERR_PARAM
    assert nslib.ns_filter_plan(10, 12, 4, 44, 152, C.byref(seg), C.byref(blocks)) == L.NS_ERR_PARAM
