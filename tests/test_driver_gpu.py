"""The program around the step on the GPU: device-side init of the dados.in
case, the output path (vorticity, contorno files), the probe recorder and
the euler.f90 time loop, against the oracle driven by a Python restatement
of euler.f90:123-169."""
import subprocess

import numpy as np
import pytest

from parity import assert_parity
from test_dados import DADOS
from navierstokes_gb300 import _lib as L

pytestmark = pytest.mark.gpu

# a 64x48 grid, 13 steps, dumps every 5 steps and probes every 2
SMALL = (DADOS.replace("imax    = 97", "imax    = 64").replace("jmax    = 81", "jmax    = 48")
         .replace("maxit   = 40", "maxit   = 12").replace("cgd     = 10", "cgd     = 5")
         .replace("D       = 12", "D       = 10"))


def small():
    from navierstokes_gb300.driver import parse_dados
    return parse_dados(SMALL)


def test_device_init_is_base_flow(nslib):
    from navierstokes_gb300.driver import solver_from_dados
    d = small()
    with solver_from_dados(d, nk=5) as s:
        U = s.get_state()
        assert np.array_equal(U, s.case.Ub)     # U = Ub (init.f90:376-384)


@pytest.mark.parametrize("nk", [5, 4])
def test_dados_case_matches_oracle(nslib, oracle_mod, nk):
    from navierstokes_gb300.driver import solver_from_dados
    d = small()
    with solver_from_dados(d, nk=nk) as s:
        s.step(0, 8)
        got = s.get_state()
        c = s.case
    ref = c.U0.copy()
    oracle_mod.Oracle(c).run(ref, 0, 8)
    assert np.abs(ref - c.Ub).max() > 1e-6      # the source has acted
    assert_parity(got, ref, c.Ub, label=f"dados.in case nk={nk}")


def test_vorticity_matches_oracle(nslib, oracle_mod):
    from navierstokes_gb300.driver import solver_from_dados, vorticity
    d = small()
    with solver_from_dados(d) as s:
        s.step(0, 5)
        U = s.get_state()
        om = vorticity(s)
        c = s.case
    ref = oracle_mod.vorticity(U, c.dm, c.dn)
    # same state in; the two differ only in the rounding of (a/h)*u vs (a*u)/h
    assert np.abs(om - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs(ref).max() > 1.0                # the mixing layer's shear


def test_probe_recorder(nslib):
    from navierstokes_gb300.driver import ProbeRecorder, dados_grid, solver_from_dados
    d = small()
    pts = dados_grid(d)["probes"]
    pi = [p[0] for p in pts]
    pj = [p[1] for p in pts]
    with solver_from_dados(d) as s:
        rec = ProbeRecorder(s, pts, capacity=5)
        want = []
        for k in range(5):
            s.step(k, 1)
            rec.capture()
            want.append(s.probes(pi, pj))
        with pytest.raises(L.NsError) as e:
            rec.capture()                         # full
        assert e.value.code == L.NS_ERR_STATE
        got = rec.drain()
        assert got.shape == (5, 3, 5)
        assert np.array_equal(got, np.array(want))
        assert rec.drain().shape[0] == 0


def euler_loop_reference(d, oracle_mod):
    """euler.f90:123-169 with the oracle's rk_euler: the probe records and
    the states dumped at each output."""
    from navierstokes_gb300.driver import dados_case, dados_grid
    c = dados_case(d, 5)
    g = dados_grid(d)
    o = oracle_mod.Oracle(c)
    U = c.U0.copy()
    cg = ct = icount = 0
    probes = [[], [], []]
    dumps = []
    for it in range(d.maxit + 1):
        t = (it + 1) * d.dt
        o.run(U, it, 1)
        if cg == d.cgd:
            dumps.append((icount, U.copy()))
            icount += 1
            cg = 0
        if ct == d.ctd:
            for q, (pi, pj) in enumerate(g["probes"]):
                probes[q].append([t] + list(U[pj - 1, pi - 1, :4]))
            ct = 0
        cg += 1
        ct += 1
    return c, probes, dumps


def test_run_euler_matches_oracle_loop(nslib, oracle_mod, tmp_path):
    from navierstokes_gb300.driver import read_dados, run_euler
    path = tmp_path / "dados.in"
    path.write_text(SMALL)
    out = tmp_path / "out"
    run_euler(path, out, nk=5)
    d = read_dados(path)
    c, probes, dumps = euler_loop_reference(d, oracle_mod)
    scale = np.array([1.0, 1.0, 1.0, 1.0])
    for q in range(3):
        got = np.loadtxt(out / f"temp{q + 1}_D60.dat", ndmin=2)
        want = np.array(probes[q])
        assert got.shape == want.shape
        assert np.array_equal(got[:, 0], want[:, 0])            # t, 17 digits round-trip
        assert np.abs(got[:, 1:] - want[:, 1:]).max() <= 1e-12 * scale.max()
    files = sorted(p.name for p in out.glob("contorno_*.dat"))
    assert files == sorted(f"contorno_{k}.dat" for k, _ in dumps)
    for k, Uref in dumps:
        text = (out / f"contorno_{k}.dat").read_text()
        lines = text.split("\n")
        # jmax records, then an empty record, for every i
        blocks = text.split("\n\n")
        assert len([b for b in blocks if b.strip()]) == d.imax
        recs = [ln for ln in lines if ln.strip()]
        assert len(recs) == d.imax * d.jmax
        assert all(len(ln) == 8 * 26 for ln in recs[:50])
        data = np.loadtxt(out / f"contorno_{k}.dat")
        I, J = np.meshgrid(np.arange(d.imax), np.arange(d.jmax), indexing="ij")
        assert np.array_equal(data[:, 0], c.m[I.ravel()])
        assert np.array_equal(data[:, 1], c.n[J.ravel()])
        ref = Uref[J.ravel(), I.ravel(), :]
        assert np.abs(data[:, 2:6] - ref[:, :4]).max() <= 1e-12
        assert np.abs(data[:, 7] - ref[:, 4]).max() <= 1e-12
        om = oracle_mod.vorticity(Uref, c.dm, c.dn)[J.ravel(), I.ravel()]
        assert np.abs(data[:, 6] - om).max() <= 1e-10 * np.abs(om).max()


def test_ns_euler_executable(nslib, tmp_path):
    from navierstokes_gb300.driver import DRIVER_PATH
    (tmp_path / "dados.in").write_text(SMALL)
    r = subprocess.run([str(DRIVER_PATH), "--maxit", "5"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Tref" in r.stdout and "Normal end of execution" in r.stdout
    assert "Tempo :" in r.stdout                   # the output at iter = cgd = 5
    assert (tmp_path / "contorno_0.dat").exists()
    assert len((tmp_path / "temp1_D60.dat").read_text().splitlines()) == 2   # iter 2, 4
    r = subprocess.run([str(DRIVER_PATH), "missing.in"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 1 and "cannot open" in r.stderr
