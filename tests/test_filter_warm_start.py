"""The two-phase warm start of the FP64 filter pieces, emulated on the CPU
(ns_kernels.cu filter_piece; ns_coef.h warmup, fp64_warmups): a piece that
starts inside a line re-runs the in-place pass-2 recurrence (filtering.f90:
69-79) from unfiltered history warm points earlier, the first warm32 steps in
FP32 and the rest in FP64, and its outputs then equal those of the serial
FP64 sweep (the C oracle's) to rounding, while a warm-up that stops early or
never leaves FP32 does not."""
import numpy as np
import pytest

SIGMAF = 0.2


def warmup(sigmaf, df, thresh, floor):
    """ns_coef.h warmup(): the last point at which the response of the
    homogeneous recurrence to any unit history is >= thresh, plus 8."""
    worst = 0
    for u in range(6):
        e = [0.0] * (4096 + 6)
        e[u] = 1.0
        last = 0
        for q in range(6, len(e)):
            v = sum(-sigmaf * df[s] * e[q - s] for s in range(1, 7))
            e[q] = v
            if abs(v) >= thresh:
                last = q - 5
        worst = max(worst, last)
    return max(floor, worst + 8)


def serial_sweep(oracle_mod, u):
    """The oracle's serial FP64 x sweep (passes 1, 2, 3) of the line u."""
    from navierstokes_gb300 import cases
    c = cases.acoustic_pulse_case(imax=len(u), jmax=16, nk=4, D=0, sigmaf=SIGMAF)
    o = oracle_mod.Oracle(c)
    U = np.zeros((c.jmax, c.imax, 4))
    U[5, :, 0] = u
    return o.filterx(U)[5, :, 0]


def warm_piece(u, a, b, warm, warm32, c0, m):
    """Outputs a..b-1 of a piece started warm points early from unfiltered
    history: warm32 steps in FP32, then FP64."""
    w = [float(x) for x in u[a - warm - 6:a - warm + 7]]
    q = a - warm
    c0f, mf = np.float32(c0), [np.float32(x) for x in m]
    wf = [np.float32(x) for x in w]
    for _ in range(warm32):
        v = c0f * wf[6] + sum(mf[k] * (wf[6 - k] + wf[6 + k]) for k in range(1, 7))
        wf = wf[1:6] + [np.float32(v)] + wf[7:] + [np.float32(u[q + 7])]
        q += 1
    w = [float(x) for x in wf]
    out = []
    while q < b:
        v = c0 * w[6] + sum(m[k] * (w[6 - k] + w[6 + k]) for k in range(1, 7))
        if q >= a:
            out.append(v)
        w = w[1:6] + [v] + w[7:] + [float(u[q + 7])]
        q += 1
    return np.array(out)


@pytest.fixture(scope="module")
def setup(oracle_mod):
    df = oracle_mod.coeffs(7)[6:]  # df(0..6)
    c0 = 1.0 - SIGMAF * df[0]
    m = [0.0] + [-SIGMAF * df[s] for s in range(1, 7)]
    w32 = warmup(SIGMAF, df, 2.0 ** -24, 0)
    w64 = warmup(SIGMAF, df, 2.0 ** -36, 16)
    return df, c0, m, w32, w32 + w64


def test_warmup_lengths(setup):
    _, _, _, w32, warm = setup
    assert (w32, warm) == (20, 48)


@pytest.mark.parametrize("seed", [0, 1])
def test_two_phase_warm_start_matches_the_serial_sweep(oracle_mod, setup, seed):
    df, c0, m, w32, warm = setup
    rng = np.random.default_rng(seed)
    n = 400
    x = np.arange(n)
    # a smooth field with unit-size noise: the worst case for the history
    u = np.sin(0.05 * x) + rng.standard_normal(n)
    ref = serial_sweep(oracle_mod, u)
    scale = np.abs(ref).max()
    for a in (120, 200, 333):
        got = warm_piece(u, a, a + 40, warm, w32, c0, m)
        assert np.abs(got - ref[a:a + 40]).max() <= 4e-16 * scale * 8
    # stopping after the FP32 phase, or an FP64 phase far too short, leaves
    # the FP32 rounding in the outputs
    short = warm_piece(u, 200, 240, w32 + 2, w32, c0, m)
    fp32_only = warm_piece(u, 200, 240, warm, warm, c0, m)
    assert np.abs(short - ref[200:240]).max() > 1e-10 * scale
    assert np.abs(fp32_only - ref[200:240]).max() > 1e-10 * scale
