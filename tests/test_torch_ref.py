"""The PyTorch FP64 restatement of the Euler step (oracle/torch_ref.py), the
reference gradient of the adjoint tests, against the C oracle (no GPU)."""
import numpy as np
import torch

from navierstokes_gb300.adjoint import SourceProblem


def test_torch_ref_step_matches_oracle(oracle_mod):
    from oracle import torch_ref as tr
    pb = SourceProblem(n=40, D=8, envelope_cells=5.0, radius=8.0, nobs=8, steps=3)
    c = pb.case
    P = tr.params(c)
    U = torch.as_tensor(np.moveaxis(c.U0, 2, 0).copy())
    S = torch.as_tensor(c.src_field)
    for n in range(3):
        U = tr.step(U, S, 4 + n, P)
    ref = c.U0.copy()
    oracle_mod.Oracle(c).run(ref, 4, 3)
    got = np.moveaxis(U.numpy(), 0, 2)
    # same statements, different summation order: a few ulps of O(1) values
    assert np.abs(got - ref).max() <= 1e-14
    assert np.abs(ref - c.Ub).max() > 1e-5     # the source did act


def test_torch_ref_gradient_is_linear_in_loss_weight(oracle_mod):
    from oracle import torch_ref as tr
    pb = SourceProblem(n=32, D=6, envelope_cells=4.0, radius=6.0, nobs=4, steps=2)
    c = pb.case
    L1, g1, _ = tr.loss_and_grad(c, c.src_field, pb.obs_x, pb.obs_y, 2)
    L2, g2, _ = tr.loss_and_grad(c, 2.0 * c.src_field, pb.obs_x, pb.obs_y, 2)
    # p' is nearly linear in S at these amplitudes: L scales by ~4, dL/dS by ~2
    assert abs(L2 / L1 - 4.0) < 1e-2
    assert np.abs(g2 - 2.0 * g1).max() < 1e-2 * np.abs(g1).max()
