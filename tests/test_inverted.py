"""ARAP constraint values and gradients of inverted tets (det F <= 0).

The reference evaluates C = |F - R|_F with R = U V^T from `ti.svd(F)`
(cons/mgpbd_gpu.py:225-247, gradient cons/mgpbd.py:35-68).  Its SVD returns
proper rotations U and V (det = +1) and carries the sign of det F on the
smallest singular value, so an inverted tet has one negative singular value
and R stays a rotation: C = sqrt(sum (s_i - 1)^2) over the SIGNED singular
values.  The CUDA `svd3_rv` (csrc/svd3.cuh) keeps that convention, and so
does the oracle's float64 `svd_rv`.

Known answer: F = diag(2, 1.5, -0.5) gives C = sqrt(1 + 0.25 + 2.25) =
sqrt(3.5) (the unsigned convention would give sqrt(1.5)), dC/dF = (F - I)/C.
Then the GPU and the oracle agree on bodies with a uniform inverting map, a
random inverting map per body, and a jittered body whose tets around a
pushed-through vertex invert.  Maps with sigma_2 + sigma_3 = 0 (R not unique,
the gradient undefined) are avoided by construction.
"""

import numpy as np
import pytest

from controllable_pbd_3d_gb300 import meshgen
from oracle import mgpbd_oracle as MO

DT = 1.0 / 300


def np_(t):
  return t.detach().cpu().numpy()


def solver(torch, xr, t):
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  invm = np.ones(len(xr), np.float32)
  x = torch.tensor(xr, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], DT, mu=1e5)
  s.init()
  return s, x


def evaluate(torch, s, x, pos):
  with torch.no_grad():
    x.copy_(torch.tensor(pos, device='cuda'))
  s._compute_C_and_gradC()
  return np_(s.constraints).astype(np.float64), np_(s.gradC).astype(np.float64)


def oracle(xr, t, pos):
  dm, _, _ = MO.rest_shape(xr, t, 1e5, DT, np.float32)
  c, g = MO.constraints(pos, t, dm, np.float32)
  F = MO.deformation(pos, t, dm, np.float64)
  return np.asarray(c, np.float64), np.asarray(g, np.float64), np.linalg.det(F)


def grid(n=3):
  xr, t = meshgen.hex_grid_tets(n, n, n, h=1.0 / n)
  return xr.astype(np.float32), t


@pytest.mark.gpu
def test_known_answer_signed_singular_value(cuda):
  torch = cuda
  xr, t = grid(2)
  s, x = solver(torch, xr, t)
  F = np.diag([2.0, 1.5, -0.5])
  pos = (xr.astype(np.float64) @ F.T).astype(np.float32)
  c, g = evaluate(torch, s, x, pos)
  np.testing.assert_allclose(c, np.sqrt(3.5), rtol=1e-5)
  # dC/dx of vertex a = column sums of (dC/dF) Dm^-T; with dC/dF = (F - I)/C
  dm, _, _ = MO.rest_shape(xr, t, 1e5, DT, np.float64)
  P = (F - np.eye(3)) / np.sqrt(3.5)
  H = P[None] @ np.swapaxes(dm, 1, 2)  # (nt, 3, 3): columns = vertices 1..3
  want = np.concatenate([-H.sum(axis=2)[:, None, :], np.swapaxes(H, 1, 2)], axis=1)
  assert np.abs(g - want).max() <= 1e-4 * np.abs(want).max()


def random_inverting_map(rng):
  """A map with det < 0 and well-separated singular values: rotations
  around diag(s) with s_3 < 0 and s_2 + s_3 far from zero."""
  q1, _ = np.linalg.qr(rng.standard_normal((3, 3)))
  q2, _ = np.linalg.qr(rng.standard_normal((3, 3)))
  q1 *= np.sign(np.linalg.det(q1))
  q2 *= np.sign(np.linalg.det(q2))
  sv = np.array([1.6, 1.1, -0.4]) * (1 + 0.1 * rng.random(3))
  return q1 @ np.diag(sv) @ q2.T


@pytest.mark.gpu
@pytest.mark.parametrize('case', ['uniform', 'random-maps', 'pushed-vertex'])
def test_inverted_tets_match_the_oracle(cuda, case):
  torch = cuda
  rng = np.random.default_rng(7)
  xr, t = grid(3)
  s, x = solver(torch, xr, t)
  if case == 'uniform':
    pos = (xr.astype(np.float64) @ np.diag([1.3, 0.9, -0.7]).T).astype(np.float32)
  elif case == 'random-maps':
    pos = (xr.astype(np.float64) @ random_inverting_map(rng).T).astype(np.float32)
  else:
    # push an interior vertex through the opposite faces of its tets
    pos = xr.astype(np.float64) + 0.01 * rng.standard_normal(xr.shape)
    centre = np.argmin(np.abs(xr - 0.5).sum(axis=1))  # an interior vertex
    pos[centre] += 0.8 * np.array([0.55, 0.45, 0.5])  # 13 of 135 tets invert
    pos = pos.astype(np.float32)
  c, g = evaluate(torch, s, x, pos)
  co, go, det = oracle(xr, t, pos)
  inv = det < 0
  assert inv.sum() >= 1
  if case != 'pushed-vertex':
    assert inv.all()
  # well-conditioned R only (sigma_2 + sigma_3 away from zero): the other
  # tets' gradients depend on an arbitrary rotation choice
  F = MO.deformation(pos, t, MO.rest_shape(xr, t, 1e5, DT, np.float32)[0], np.float64)
  _, sv, _ = MO.svd_rv(F)
  ok = np.abs(sv[:, 1] + sv[:, 2]) > 0.05
  assert ok[inv].sum() >= 1
  assert np.abs(c - co).max() <= 1e-5 * max(np.abs(co).max(), 1.0)
  assert np.abs(g[ok] - go[ok]).max() <= 1e-4 * np.abs(go[ok]).max()
