"""Discrete adjoint of the FP64 Euler step (ns_adjoint_*): gradient of the
observer loss with respect to the source field, against PyTorch FP64
autograd through oracle/torch_ref.py and against central finite
differences (GPU)."""
import numpy as np
import pytest

from oracle import torch_ref
from navierstokes_gb300.adjoint import Adjoint, SourceProblem, source_loss_function

pytestmark = pytest.mark.gpu

# Tolerances.  The loss and the adjoint seeds 2*p' are built from
# p' = p - p_b ~ 1e-4 taken out of O(1) state values, so the two forward runs'
# rounding (~1e-15 absolute, different summation orders) is ~1e-11 of p':
# losses and gradient fields agree to L_RTOL and GRAD_RTOL relative.  Central
# differences with h = 1e-7 on controls of size 1e-3: truncation O(h^2) and
# rounding noise well below FD_RTOL.
L_RTOL = 1e-9
GRAD_RTOL = 1e-9
FD_RTOL = 1e-6


def small_problem(n=40, steps=5, **kw):
    kw.setdefault("D", 8)
    kw.setdefault("envelope_cells", 5.0)
    kw.setdefault("radius", 8.0)
    kw.setdefault("nobs", 8)
    return SourceProblem(n=n, steps=steps, **kw)


def rel_field_err(g, ref):
    return float(np.abs(g - ref).max() / np.abs(ref).max())


@pytest.mark.parametrize("K", [0, 1, 2, 5])
def test_adjoint_matches_torch_autograd(nslib, oracle_mod, K):
    # K = 0: every stage input kept, only first derivatives recomputed
    pb = small_problem(steps=5)
    S = pb.case.src_field
    L_ref, g_ref, _ = torch_ref.loss_and_grad(pb.case, S, pb.obs_x, pb.obs_y, 5)
    with Adjoint(pb, checkpoint_every=K) as adj:
        adj.set_field(S)
        L = adj.forward(5)
        assert (adj.stored_bytes() > 0) == (K == 0)
        g = adj.backward()
    assert abs(L - L_ref) <= L_RTOL * abs(L_ref), (L, L_ref)
    err = rel_field_err(g, g_ref)
    print(f"K={K}: gradient error {err:.3e}, loss {abs(L - L_ref) / L_ref:.3e}")
    assert err <= GRAD_RTOL, f"K={K}: max|g - g_ref|/max|g_ref| = {err:.3e}"


def test_checkpoint_intervals_give_identical_gradients(nslib):
    """Every storage mode runs the same kernels on the same stage inputs, so
    the gradient is the same bit for bit: every stage kept (K = 0), one
    segment (K = 7), and segments whose recompute runs beside the reverse of
    the next one (K = 2, 3; the last segment partial and kept by the forward).
    A second backward after one forward recomputes every segment and gives
    the same bits again."""
    pb = small_problem(n=48, steps=7, nobs=6)
    S = pb.case.src_field
    grads = {}
    for K in (0, 7, 3, 2):
        with Adjoint(pb, checkpoint_every=K) as adj:
            adj.set_field(S)
            adj.forward(7, iter0=2)
            grads[K] = adj.backward()
            if K == 2:
                again = adj.backward()
                assert np.array_equal(again, grads[K])
    for K in (7, 3, 2):
        assert np.array_equal(grads[K], grads[0]), K


def test_adjoint_nonzero_iter0_faster_mean_flow(nslib, oracle_mod):
    # iter0 shifts the source phase sin(wf*(iter+c_k)*dt); M = 0.5
    pb = small_problem(n=48, steps=4, mach=0.5, omega=0.9, radius=10.0, nobs=5)
    S = pb.case.src_field
    L_ref, g_ref, _ = torch_ref.loss_and_grad(pb.case, S, pb.obs_x, pb.obs_y, 4, iter0=11)
    with Adjoint(pb, checkpoint_every=3) as adj:
        adj.set_field(S)
        L = adj.forward(4, iter0=11)
        g = adj.backward()
    assert abs(L - L_ref) <= L_RTOL * abs(L_ref), (L, L_ref)
    err = rel_field_err(g, g_ref)
    print(f"gradient error {err:.3e}, loss {abs(L - L_ref) / L_ref:.3e}")
    assert err <= GRAD_RTOL, err


def test_adjoint_forward_leaves_solver_state(nslib, oracle_mod):
    # the forward pass is the plain FP64 step: its end state is the oracle's
    import ctypes as C
    from navierstokes_gb300 import _lib as L
    pb = small_problem(steps=6)
    c = pb.case
    with Adjoint(pb, checkpoint_every=4) as adj:
        adj.set_field(c.src_field)
        adj.forward(6, iter0=2)
        adj.backward()
        ctx = C.c_void_p()
        L.check(adj.lib.ns_adjoint_context(adj._h, C.byref(ctx)))
        got = np.empty(c.U0.shape)
        L.check(adj.lib.ns_get_state(ctx, got.ctypes.data, L.NS_LAYOUT_FORTRAN))
    ref = c.U0.copy()
    oracle_mod.Oracle(c).run(ref, 2, 6)
    from parity import assert_parity
    assert_parity(got, ref, c.Ub, label="adjoint forward end state")


def test_adjoint_finite_differences_small(nslib):
    # On this 40x40 grid p' at the observers is ~1e-5 and the change of p'
    # over +-h is ~1e-9 of an O(1) state, so the differences carry ~1e-6 of
    # rounding noise relative to max|grad|: the check is against max|grad|.
    pb = small_problem(steps=8)
    h = 1e-7
    with Adjoint(pb, checkpoint_every=3) as adj:
        _, gc = adj.loss_and_grad(pb.controls, 8)
        gmax = np.abs(gc).max()
        for (a, b) in [(7, 7), (8, 6), (6, 9), (9, 8)]:
            cp = pb.controls.copy()
            cp[a, b] += h
            adj.set_field(pb.field(cp))
            Lp = adj.forward(8)
            cp[a, b] -= 2 * h
            adj.set_field(pb.field(cp))
            Lm = adj.forward(8)
            fd = (Lp - Lm) / (2 * h)
            print(f"control ({a},{b}): adjoint {gc[a, b]:.12e} fd {fd:.12e} "
                  f"rel {abs(fd - gc[a, b]) / abs(gc[a, b]):.2e}")
            assert abs(fd - gc[a, b]) <= 1e-5 * gmax, (a, b, fd, gc[a, b], gmax)


def test_autograd_function(nslib):
    import torch
    pb = small_problem(steps=6)
    with Adjoint(pb, checkpoint_every=2) as adj:
        _, gc = adj.loss_and_grad(pb.controls, 6)
        fn = source_loss_function()
        x = torch.tensor(pb.controls, dtype=torch.float64, requires_grad=True)
        loss = fn.apply(x, adj, 6)
        (2.5 * loss).backward()
    assert np.allclose(x.grad.numpy(), 2.5 * gc, rtol=1e-13, atol=0.0)


def test_adjoint_full_grid_chunked_filters(nslib, oracle_mod):
    """512x512 (two chunks per filter line): 2 steps against autograd."""
    pb = SourceProblem(n=512, steps=2, radius=20.0, nobs=8)
    S = pb.case.src_field
    L_ref, g_ref, _ = torch_ref.loss_and_grad(pb.case, S, pb.obs_x, pb.obs_y, 2)
    with Adjoint(pb, checkpoint_every=1) as adj:
        adj.set_field(S)
        L = adj.forward(2)
        g = adj.backward()
    assert abs(L - L_ref) <= L_RTOL * abs(L_ref), (L, L_ref)
    err = rel_field_err(g, g_ref)
    print(f"gradient error {err:.3e}, loss {abs(L - L_ref) / L_ref:.3e}")
    assert err <= GRAD_RTOL, err


@pytest.mark.slow
def test_source_problem_finite_differences(nslib):
    """The 512x512, 2000-step source problem: the control gradient at two
    controls near the source against central differences, h = 1e-7."""
    pb = SourceProblem()
    h = 1e-7
    with Adjoint(pb, checkpoint_every=100) as adj:
        L0, gc = adj.loss_and_grad(pb.controls)
        assert np.isfinite(L0) and L0 > 0
        for (a, b) in [(7, 8), (8, 7)]:
            cp = pb.controls.copy()
            cp[a, b] += h
            adj.set_field(pb.field(cp))
            Lp = adj.forward()
            cp[a, b] -= 2 * h
            adj.set_field(pb.field(cp))
            Lm = adj.forward()
            fd = (Lp - Lm) / (2 * h)
            print(f"control ({a},{b}): adjoint {gc[a, b]:.12e} fd {fd:.12e} "
                  f"rel {abs(fd - gc[a, b]) / abs(gc[a, b]):.2e}")
            assert abs(fd - gc[a, b]) <= FD_RTOL * abs(gc[a, b]), (a, b, fd, gc[a, b])
