"""The stiff-drag scenario (a slab with one long edge pinned, the opposite
corner dragged along +z by a moving kinematic target): mesh and driver
(CPU), and on the GPU a reduced slab dragged over a few frames with the
length + volume constraints."""

import numpy as np
import pytest

from controllable_pbd_3d_gb300.scenarios import drag_slab, grid_edge_vertices


def test_drag_slab_layout():
  s = drag_slab(6, 2, 5)
  xr = s['x_ref']
  assert len(xr) == 7 * 3 * 6 and len(s['t_i']) == 4 * 5 * 6 * 2 * 5
  # the pinned edge lies on y = 0, z = 0 along x; the dragged corner at max
  assert np.allclose(xr[s['pinned'], 1], 0) and np.allclose(xr[s['pinned'], 2], 0)
  assert np.ptp(xr[s['pinned'], 0]) == pytest.approx(xr[:, 0].max())
  assert np.allclose(xr[s['drag']], xr.max(axis=0))
  assert (s['invm'][s['pinned']] == 0).all() and s['invm'][s['drag']] == 0
  assert (s['invm'] > 0).sum() == len(xr) - len(s['pinned']) - 1
  assert list(grid_edge_vertices(3, 1, 1)) == [0, 1, 2, 3]


@pytest.mark.gpu
def test_gpu_drag_follows_the_target(cuda):
  torch = cuda
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  from controllable_pbd_3d_gb300.scenarios import DragDriver
  s = drag_slab(12, 3, 12, h=1.0 / 12)
  x = torch.tensor(s['x0'], device='cuda')
  solver = MGPBDSolverGPU(x, torch.tensor(s['x_ref'], device='cuda'),
                          torch.tensor(s['invm'], device='cuda'),
                          torch.tensor(s['t_i'], device='cuda'), None, [0.0, -9.8, 0.0], 1 / 300,
                          constraints='edge_volume', compliance=1e-8, kinematic_pins=True,
                          mode='fast', precond='cheb', primal=True, rel_tol_cg=1e-6,
                          tol_cg=1e-12, maxiter_cg=4000)
  solver.init()
  frames = 6
  drv = DragDriver(solver, s['drag'], distance=0.2, frames=frames)
  for f in range(frames):
    drv.frame(f, substeps=2)
    st = solver.stats()
    assert not (st['status'] & 1), st  # no NaN
  xn = x.cpu().numpy()
  assert np.isfinite(xn).all()
  # the dragged vertex sits on its last target, the pinned edge has not moved
  assert np.allclose(xn[s['drag']], drv.target(frames - 1).cpu().numpy(), atol=1e-6)
  assert np.array_equal(xn[s['pinned']], s['x0'][s['pinned']])
  # the body followed: the free vertex next to the dragged corner moved up in z
  near = s['drag'] - 1
  assert xn[near, 2] - s['x0'][near, 2] > 0.05


def test_training_bodies_follow_the_configuration():
  """Seeded training bodies: side counts in 20..40, half of them projected
  onto a ball, compliance log-uniform in [1e-9, 1e-4], 1-4 % of the
  surface vertices pinned."""
  from controllable_pbd_3d_gb300 import meshgen
  from controllable_pbd_3d_gb300.scenarios import grid_surface_vertices, training_bodies
  bodies = list(training_bodies(6, seed=3))
  again = list(training_bodies(6, seed=3))
  for b, c in zip(bodies, again):
    assert np.array_equal(b['x0'], c['x0']) and np.array_equal(b['pinned'], c['pinned'])
    n = b['side']
    assert 20 <= n <= 40
    assert len(b['x_ref']) == (n + 1) ** 3 and len(b['t_i']) == 4 * 5 * n ** 3
    assert 1e-9 <= b['compliance'] <= 1e-4
    surf = grid_surface_vertices(n, n, n)
    assert np.isin(b['pinned'], surf).all()
    frac = len(b['pinned']) / len(surf)
    assert 0.01 - 1 / len(surf) <= frac <= 0.04 + 1 / len(surf)
    assert (b['invm'] == 0).sum() == len(b['pinned'])
    xr = b['x_ref'].astype(np.float64)
    c0 = 0.5 * (xr.min(axis=0) + xr.max(axis=0))
    r = np.linalg.norm(xr - c0, axis=1)
    if b['ball']:
      assert r.max() <= 0.5 + 1e-5  # the unit cube's inscribed ball
    else:
      assert r.max() == pytest.approx(0.5 * np.sqrt(3), rel=1e-5)
  assert {b['ball'] for b in bodies} == {True, False}
  x, t = meshgen.hex_grid_tets(4, 4, 4)
  assert np.array_equal(grid_surface_vertices(4, 4, 4), meshgen.surface_vertices(t))


@pytest.mark.gpu
def test_gpu_training_over_several_bodies_lowers_the_loss(cuda):
  """Pairs from two seeded training bodies (reduced sides), recorded by the
  plain solver, then Adam steps alternating over the bodies."""
  from controllable_pbd_3d_gb300.learned import CoarseNet, train_on_bodies
  from controllable_pbd_3d_gb300.scenarios import training_bodies
  net = CoarseNet(seed=1)
  losses, data = train_on_bodies(net, training_bodies(2, seed=5, sides=(8, 10)),
                                 pairs_per_body=32, every=2, steps=200, batch=8, lr=2e-3)
  assert len(data) == 2 and all(rc.shape[0] > 0 for _, rc in data)
  assert np.isfinite(losses).all()
  assert losses[-20:].mean() < losses[:10].mean()
