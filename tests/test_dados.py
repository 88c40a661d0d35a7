"""The program around the step on the host (no GPU): the dados.in reader
(init.f90:10-52), the grid and base-flow setup (init.f90:56-210, :341-373)
against the C oracle and the Python setup, and the list-directed number
layout of the output files."""
import math
import random

import numpy as np
import pytest

from navierstokes_gb300 import _lib as L
from navierstokes_gb300 import cases

# The layout of the reference's dados.in (groups, comments, tabs, &end and
# $end terminators, the second &grid group) with values chosen here.
DADOS = """&grid
!******number of points in x direction
imax    = 97
!******number of points in y direction
jmax    = 81
!******number of temporal iteration
maxit   = 40
!******step time
dt      = 0.02d0
!******filter parameter(<0.2)
sigmaf  = 0.15d0
cgd     = 10
cfd     = 1
ctd     = 2
&end

&freq
r0_acous  = 0.25d0
amplitude = 0.5d0
m_pt_acous= 1.d0
n_pt_acous= -0.5d0
wfi       = 0.3d0
wff\t    = 2.3d0
wf \t    = 1.5d0
iterw\t    = 7
pxfft1    = 7.d0
pxfft2    = 9.d0
pxfft3    = 10.d0
pxfft4    = 18.d0
pxfft5    = 20.d0
&end

&freeadm
!*********xdomain
mmin= -4.0d0
mmax= 12.0d0
!*********ydomain
nmin= -3.2d0
nmax=  3.2d0
pxr1=  2.0d0
pyr1=  0.0d0
pxr2=  2.0d0
pyr2=  0.8d0
pxr3=  5.5d0
pyr3= -0.8d0
&end

&flow
U1 = 0.8d0
U2 = 0.2d0
Re = 5000.0d0
Pr = 0.72d0
T1 = 1.0d0
T2 = 0.6d0
Tref = 300.0d0
&end

&grid
!*********Number of points in the NRBC
D       = 12
c1b     = 0.02d0
c2b     = 15.0d0
c3b     = 40.0d0
&end

&mpi
num_procs_x=2
num_procs_y=3
$end
"""


def parse(text):
    from navierstokes_gb300.driver import parse_dados
    return parse_dados(text)


def test_reads_every_group(nslib):
    d = parse(DADOS)
    assert (d.imax, d.jmax, d.maxit, d.cgd, d.cfd, d.ctd) == (97, 81, 40, 10, 1, 2)
    assert (d.dt, d.sigmaf) == (0.02, 0.15)
    assert (d.r0_acous, d.amplitude, d.m_pt_acous, d.n_pt_acous) == (0.25, 0.5, 1.0, -0.5)
    assert (d.wfi, d.wff, d.wf, d.iterw) == (0.3, 2.3, 1.5, 7)
    assert list(d.pxfft) == [7.0, 9.0, 10.0, 18.0, 20.0]
    assert (d.mmin, d.mmax, d.nmin, d.nmax) == (-4.0, 12.0, -3.2, 3.2)
    assert list(d.pxr) == [2.0, 2.0, 5.5] and list(d.pyr) == [0.0, 0.8, -0.8]
    assert (d.U1, d.U2, d.Re, d.Pr, d.T1, d.T2, d.Tref) == (0.8, 0.2, 5000.0, 0.72, 1.0, 0.6,
                                                           300.0)
    # the second &grid group (init.f90:22 extends group grid)
    assert (d.D, d.c1b, d.c2b, d.c3b) == (12, 0.02, 15.0, 40.0)
    assert (d.num_procs_x, d.num_procs_y) == (2, 3)


def test_read_from_file(nslib, tmp_path):
    from navierstokes_gb300.driver import read_dados
    p = tmp_path / "dados.in"
    p.write_text(DADOS)
    assert read_dados(p).imax == 97


def test_separators_case_and_exponents(nslib):
    text = ("&GRID imax=33, JMAX = 29 ,maxit=5 dt=1.0D-3, sigmaf=.2d0 cgd=1 cfd=1 ctd=1 /\n"
            "&freq wf=2E0 /\n&freeadm mmin=-1 mmax=1 nmin=-1 nmax=1 /\n"
            "&flow U1=1 U2=0 /\n&grid D=4 c1b=1.e-2 c2b=20. /\n&mpi /\n")
    d = parse(text)
    assert (d.imax, d.jmax, d.maxit, d.dt, d.sigmaf) == (33, 29, 5, 1e-3, 0.2)
    assert (d.wf, d.mmin, d.U1, d.D, d.c1b, d.c2b) == (2.0, -1.0, 1.0, 4, 0.01, 20.0)


def test_groups_are_found_by_scanning_forward(nslib):
    # anything before a group (other text, other groups) is skipped
    text = "a title line\n" + DADOS.replace("&freq", "&other x=1 /\n&freq", 1)
    assert parse(text).wf == 1.5


@pytest.mark.parametrize("bad,what", [
    (DADOS.replace("cfd     = 1", "cfx     = 1"), "cfx"),             # name not in the group
    (DADOS.replace("imax    = 97", "imax    = 97.5"), "imax"),        # real for an integer
    (DADOS.replace("dt      = 0.02d0", "dt      = 0.0.2"), "dt"),     # malformed real
    (DADOS.replace("&flow", "&flaw"), "&flow"),                       # group missing
    (DADOS.replace("$end", ""), "terminator"),                        # last group unterminated
    (DADOS.replace("Re = 5000.0d0", "Re = "), "Re"),                  # no value
])
def test_errors_name_the_line(nslib, bad, what):
    from navierstokes_gb300.driver import parse_dados
    with pytest.raises(L.NsError) as e:
        parse_dados(bad)
    assert e.value.code == L.NS_ERR_PARAM
    msg = str(e.value)
    assert "line" in msg and what.lower() in msg.lower(), msg


def test_missing_file(nslib, tmp_path):
    from navierstokes_gb300.driver import read_dados
    with pytest.raises(L.NsError):
        read_dados(tmp_path / "nope.in")


@pytest.mark.parametrize("quirk", [True, False])
def test_grid_matches_oracle_and_python(nslib, oracle_mod, quirk):
    from navierstokes_gb300.driver import dados_grid
    d = parse(DADOS)
    g = dados_grid(d, quirk)
    ref = oracle_mod.init_dados(d.imax, d.jmax, d.D, d.mmin, d.mmax, d.nmin, d.nmax, d.c1b,
                                d.c2b, quirk)
    py = cases.init_dados(d.imax, d.jmax, d.D, d.mmin, d.mmax, d.nmin, d.nmax, d.c1b, d.c2b,
                          quirk)
    for k in ("m", "n", "meshx", "meshy", "sigmax", "sigmay"):
        assert np.array_equal(g[k], ref[k]), k      # same statements, same bits
        assert np.array_equal(g[k], py[k]), k
    assert (g["dm"], g["dn"]) == (ref["dm"], ref["dn"])
    # init.f90:80-85: px = int(-mmin/dm + pxr/dm + 1)
    want = [(int(-d.mmin / g["dm"] + d.pxr[q] / g["dm"] + 1),
             int(-d.nmin / g["dn"] + d.pyr[q] / g["dn"] + 1)) for q in range(3)]
    assert g["probes"] == want


def test_quirk_clamps_left_and_bottom(nslib):
    from navierstokes_gb300.driver import dados_grid
    d = parse(DADOS)
    g = dados_grid(d, True)
    assert np.all(g["sigmax"][:d.D] == 0.0) and np.all(g["sigmay"][:d.D] == 0.0)
    assert np.all(g["sigmax"][-d.D:-1] > 0.0)
    g2 = dados_grid(d, False)
    assert np.all(g2["sigmax"][1:d.D] > 0.0)


def test_profiles_match_oracle(nslib, oracle_mod):
    from navierstokes_gb300.driver import dados_grid, dados_profiles
    d = parse(DADOS)
    n = dados_grid(d)["n"]
    got = dados_profiles(d, n)
    ref = oracle_mod.mixing_layer(n, d.U1, d.U2, d.T1, d.T2)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    py = cases.mixing_layer(n, d.U1, d.U2, d.T1, d.T2)
    for a, b in zip(got, py):
        assert np.allclose(a, b, rtol=1e-15, atol=1e-15)


# ---------------------------------------------------------------------------
# List-directed REAL(8) items: G25.17 with a three-digit exponent.
# ---------------------------------------------------------------------------

def listdirected(x: float) -> str:
    """The layout rules, restated: 17 significant digits rounded once; for
    0.1 <= |x| < 1e17 (after rounding) and for 0, F20.(16-e) right-justified
    plus five blanks; otherwise one digit, the point, 16 digits, E, sign and
    three exponent digits, right-justified in 25."""
    if math.isnan(x):
        return "NaN".rjust(25)
    if math.isinf(x):
        return ("Infinity" if x > 0 else "-Infinity").rjust(25)
    sign = "-" if math.copysign(1.0, x) < 0 else ""
    a = abs(x)
    if a == 0.0:
        return (sign + "0." + "0" * 16).rjust(20) + " " * 5
    mant, exp = f"{a:.16e}".split("e")
    e = int(exp)
    if -1 <= e <= 16:
        dec = 16 - e
        body = sign + f"{a:.{dec}f}" + ("." if dec == 0 else "")
        return body.rjust(20) + " " * 5
    return (sign + mant + "E" + ("-" if e < 0 else "+") + f"{abs(e):03d}").rjust(25)


@pytest.mark.parametrize("x,want", [
    (1.0, "  1.0000000000000000     "),
    (0.1, " 0.10000000000000001     "),
    (-2.5, " -2.5000000000000000     "),
    (0.0, "  0.0000000000000000     "),
    (123.456, "  123.45600000000000     "),
    (1e-5, "  1.0000000000000001E-005"),
    (1e20, "  1.0000000000000000E+020"),
    (-3.3e-200, " -3.2999999999999998E-200"),
    (1e16, "  10000000000000000.     "),
])
def test_format_real_examples(nslib, x, want):
    from navierstokes_gb300.driver import format_real
    assert format_real(x) == want
    assert listdirected(x) == want


def test_format_real_random(nslib):
    from navierstokes_gb300.driver import format_real
    rnd = random.Random(7)
    for _ in range(3000):
        x = rnd.choice([-1, 1]) * 10.0 ** rnd.uniform(-30, 30)
        assert format_real(x) == listdirected(x), x
    for x in (0.09999999999999999, 0.1, 9.999999999999999e16, 1e17, float("nan"),
              float("inf"), -float("inf"), -0.0, 5e-324):
        assert format_real(x) == listdirected(x), x
