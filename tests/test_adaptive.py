"""Adaptive zones and the adaptive solver (cons/adaptive_zone.py,
cons/mgpbd_adaptive.py): zone flags bit for bit against the oracle's
restatement, and an adaptive substep against the float64 oracle stepping
with the same compliance mask."""

import numpy as np
import pytest

from controllable_pbd_3d_gb300 import meshgen


def _cube(n, seed=5, jitter=0.02):
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=jitter, seed=seed)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  return xr, x0, t, invm


@pytest.mark.parametrize('n,jitter', [(3, 0.0), (5, 0.03)])
def test_host_face_adjacency_matches_oracle(n, jitter):
  from controllable_pbd_3d_gb300.adaptive import host_face_adjacency
  from oracle.mgpbd_oracle import face_adjacency_sets
  _, _, t, _ = _cube(n, jitter=jitter)
  nt = len(t) // 4
  ip, ix = host_face_adjacency(t, nt)
  adj = face_adjacency_sets(t, nt)
  for k in range(nt):
    assert list(ix[ip[k]:ip[k + 1]]) == sorted(adj[k])


@pytest.mark.gpu
def test_zone_kernels_match_oracle(cuda):
  from controllable_pbd_3d_gb300.adaptive import AdaptiveZone
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  from oracle.mgpbd_oracle import (face_adjacency_sets, zone_expand, zone_proximity,
                                   zone_strain)
  n = 8
  xr, x0, t, invm = _cube(n)
  nt = len(t) // 4
  x = cuda.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                     cuda.tensor(t, device='cuda'), None, [0, -9.8, 0], 1 / 300)
  s.init()
  zone = AdaptiveZone(nt, s.t_i, s.v_p, solver=s)
  adj = face_adjacency_sets(t, nt)
  rng = np.random.default_rng(0)
  for _ in range(4):
    c = rng.uniform(0.0, 1.0, 3).astype(np.float32)
    r = float(rng.uniform(0.1, 0.5))
    zone.update_by_proximity(*c, r)
    want = zone_proximity(x0, t, c, r)
    np.testing.assert_array_equal(zone.tet_active.cpu().numpy(), want)
    for rings in (1, 2):
      zone.update_by_proximity(*c, r)
      zone.expand_zone(rings)
      np.testing.assert_array_equal(zone.tet_active.cpu().numpy(), zone_expand(want, adj, rings))
  x_old = x0 + rng.normal(0.0, 1e-3, x0.shape).astype(np.float32)
  for thr in (0.05, 0.2, 0.4):
    zone.update_by_strain(cuda.tensor(x_old, device='cuda'), thr, 1 / 300)
    np.testing.assert_array_equal(zone.tet_active.cpu().numpy(),
                                  zone_strain(x0, x_old, t, thr, 1 / 300))
  assert 0.0 < zone.get_active_fraction() < 1.0


@pytest.mark.gpu
def test_adaptive_step_matches_masked_oracle_step(cuda):
  from controllable_pbd_3d_gb300.adaptive import AdaptiveZone, MGPBDAdaptiveSolver
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  from oracle.mgpbd_oracle import (MGPBDOracle, face_adjacency_sets, zone_expand,
                                   zone_proximity)
  n = 8
  xr, x0, t, invm = _cube(n, seed=2)
  nt = len(t) // 4
  kw = dict(mu=1e5, damp=0.993, maxiter=5, rtol=1e-6, atol=1e-9, maxiter_cg=400, tol_cg=1e-10,
            rel_tol_cg=1e-7)
  g, dt = [0.0, -9.8, 0.0], 1 / 300
  tool, radius = (0.9, 0.1, 0.85), 0.45
  x = cuda.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                     cuda.tensor(t, device='cuda'), None, g, dt, **kw)
  s.init()
  ad = MGPBDAdaptiveSolver(s, AdaptiveZone(nt, s.t_i, s.v_p))
  o = MGPBDOracle(x0, xr, invm, t, g, dt, dtype=np.float64, **kw)
  o.init()
  adj = face_adjacency_sets(t, nt)
  alpha0 = o.alpha.copy()
  alpha_gpu = s.alpha_tilde.cpu().numpy().copy()
  for k in range(2):
    ad.step(k, tool_pos=tool, tool_radius=radius)
    o.make_prediction()
    xp = o.x.astype(np.float32)
    # the flags must not hinge on rounding: every vertex clears the radius
    d = np.sqrt(((xp - np.asarray(tool, np.float32)) ** 2).sum(1))
    assert np.abs(d - radius).min() > 1e-4
    mask = zone_expand(zone_proximity(xp, t, tool, radius), adj, 1)
    np.testing.assert_array_equal(ad.zone.tet_active.cpu().numpy(), mask)
    assert 0 < mask.sum() < nt
    o.alpha = np.where(mask == 1, alpha0, 1e20)
    o.solve(k)
    o.alpha = alpha0.copy()
    o.update_vel()
  err = float(np.abs(x.cpu().numpy() - o.x).max())
  assert err <= 1e-5 * float(np.abs(o.x).max()), err
  np.testing.assert_array_equal(s.alpha_tilde.cpu().numpy(), alpha_gpu)  # restored


@pytest.mark.parametrize('name', ['cube5', 'box6x3x4'])
def test_oracle_zones_match_the_reference(name):
  """The oracle's zone restatement against the reference's own AdaptiveZone
  (proximity, two face rings, strain rate), bit for bit
  (`tests/golden/zone.npz`, written by `make_golden.py --only zone`)."""
  from conftest import golden
  from oracle.mgpbd_oracle import face_adjacency_sets, zone_expand, zone_proximity, zone_strain
  z = golden('zone.npz')
  g = lambda k: z[f'{name}_{k}']  # noqa: E731
  t = g('t')
  nt = len(t) // 4
  prox = zone_proximity(g('x'), t, g('center'), g('radius'))
  assert np.array_equal(prox, g('prox'))
  assert np.array_equal(zone_expand(prox, face_adjacency_sets(t, nt), 2), g('ring2'))
  assert np.array_equal(zone_strain(g('x'), g('x_old'), t, g('threshold'), g('dt')), g('strain'))


@pytest.mark.parametrize('dtype', [np.float32, np.float64])
def test_oracle_adaptive_step_matches_the_reference(dtype):
  """Two substeps of the reference's own MGPBDAdaptiveSolver
  (`tests/golden/adaptive.npz`, `make_golden.py --only adaptive`): the
  oracle, stepping with its zone flags (proximity of the predicted
  positions, one face ring) and alpha~ = 1e20 on passive tets, reproduces
  the flags bit for bit and the positions to the step fixtures' tolerance."""
  from conftest import golden, solver_kwargs
  from oracle.mgpbd_oracle import (MGPBDOracle, face_adjacency_sets, zone_expand,
                                   zone_proximity)
  z = golden('adaptive.npz')
  t = z['t_i']
  nt = len(t) // 4
  o = MGPBDOracle(z['x0'], z['x_ref'], z['invm'], t, z['gravity'], float(z['dt']), dtype=dtype,
                  **solver_kwargs(z))
  o.init()
  adj = face_adjacency_sets(t, nt)
  alpha0 = o.alpha.copy()
  for k in range(len(z['x_traj'])):
    o.make_prediction()
    mask = zone_expand(zone_proximity(o.x.astype(np.float32), t, z['tool'], z['radius']), adj, 1)
    assert np.array_equal(mask, z['masks'][k])
    o.alpha = np.where(mask == 1, alpha0, dtype(1e20)).astype(dtype)
    o.solve(k)
    o.alpha = alpha0.copy()
    o.update_vel()
    scale = float(np.abs(z['x_traj'][k]).max())
    err = float(np.abs(o.x - z['x_traj'][k]).max())
    assert err <= (2e-6 if dtype == np.float32 else 1e-5) * scale, (k, err)
  assert np.array_equal(o.alpha, alpha0)  # restored after every substep
  assert np.allclose(alpha0, z['alpha_tilde'], rtol=1e-6, atol=0)
