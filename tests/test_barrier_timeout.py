"""The persistent CG kernels' bounded grid barrier turns a wait that runs
out into an error code, and the handle keeps working.

Every grid-barrier wait of the cooperative CG kernels polls with a time
limit; a block whose wait reaches it sets the error flag and
MGPBD_STATUS_SYNC_TIMEOUT and returns, the other blocks leave at their next
wait, and the call returns MGPBD_ECUDA.  Here the limit is set to 0
(`mgpbd_set_barrier_limit`): a block gives up at the first poll that finds
another block not yet arrived, which the launch ramp of a few hundred
blocks makes certain at the first barrier.  No block withholds an arrival,
and every block ends within its first barriers: nothing can hang.
The same solve, repeated with the default limit back, must succeed and land
where an untouched solver does.
"""

import ctypes as C

import numpy as np
import pytest

from controllable_pbd_3d_gb300 import _native as N
from controllable_pbd_3d_gb300 import meshgen

SYNC_TIMEOUT = 32
ECUDA = -2


def test_barrier_limit_is_validated():
  L = N.lib()
  p = N.default_params()
  p.dt = 1.0 / 300
  h = C.c_void_p()
  N.check(L.mgpbd_create(C.byref(p), C.byref(h)), 'mgpbd_create')
  try:
    assert L.mgpbd_set_barrier_limit(h, -1.0) == -1
    assert L.mgpbd_set_barrier_limit(h, 0.0) == 0
    assert L.mgpbd_set_barrier_limit(h, 61.0) == -1
    assert L.mgpbd_set_barrier_limit(h, 4.0) == 0
    assert L.mgpbd_set_barrier_limit(None, 4.0) == -1
  finally:
    L.mgpbd_destroy(h)


def body(torch, n=6, **kw):
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=4)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  x = torch.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], 1.0 / 300,
                     constraints='edge_volume', compliance=1e-6, kinematic_pins=True,
                     mode='fast', precond='cheb', cheb_lo=1e-3, maxiter=5, rtol=1e-6,
                     atol=1e-9, maxiter_cg=3000, tol_cg=1e-12, rel_tol_cg=1e-7, **kw)
  s.init()
  return s, x


@pytest.mark.gpu
@pytest.mark.parametrize('variant', [dict(primal=False), dict(primal=True, primal_tol=1e-2),
                                     dict(primal=False, persistent=2)])
def test_barrier_timeout_is_an_error_and_the_handle_recovers(cuda, variant):
  from controllable_pbd_3d_gb300._native import MGPBDError
  torch = cuda
  L = N.lib()
  s, x = body(torch, **variant)
  ref, xr = body(torch, **variant)
  s.step(0)
  ref.step(0)
  assert L.mgpbd_set_barrier_limit(s._h, 0.0) == 0
  s.make_prediction()
  x_before = x.clone()
  with pytest.raises(MGPBDError) as e:
    s.solve(1)
  assert e.value.code == ECUDA
  assert 'timed out' in str(e.value)
  st = C.c_uint32()
  N.check(L.mgpbd_get_status(s._h, C.byref(st)), 'mgpbd_get_status')
  assert st.value & SYNC_TIMEOUT
  torch.cuda.synchronize()
  assert L.mgpbd_set_barrier_limit(s._h, 4.0) == 0
  # the same solve again from the predicted positions, then a full
  # substep: both must succeed
  with torch.no_grad():
    x.copy_(x_before)
  s.solve(1)
  s.update_vel()
  ref.step(1)
  assert s.stats()['status'] & SYNC_TIMEOUT == 0
  assert torch.isfinite(x).all()
  assert float((x - xr).abs().max()) <= 1e-5 * float(xr.abs().max())
  s.step(2)
  ref.step(2)
  assert float((x - xr).abs().max()) <= 1e-5 * float(xr.abs().max())


@pytest.mark.gpu
def test_barrier_timeout_in_the_captured_body_substep(cuda):
  """Packed bodies, substep as one captured graph: a persistent CG launch
  inside the graph whose barrier wait runs out ends the device-side Newton
  loop, the call returns MGPBD_ECUDA with MGPBD_STATUS_SYNC_TIMEOUT, and
  with the limit back the graph is captured again and the same solve lands
  where an untouched batch does."""
  from controllable_pbd_3d_gb300._native import MGPBDError
  from controllable_pbd_3d_gb300.batch import BodyBatch, random_bodies
  torch = cuda
  L = N.lib()
  kw = dict(mode='fast', precond='cheb', cheb_scale='none', cheb_lo=1e-3, primal=False,
            rel_tol_cg=1e-7, tol_cg=1e-14, maxiter_cg=3000, maxiter=5, atol=1e-9, rtol=3e-3,
            kinematic_pins=True, constraints='edge_volume')
  bodies = random_bodies(3, seed=5, dims=(3, 6), compliance=(1e-7, 1e-5))
  g, dt = [0.0, -9.8, 0.0], 1.0 / 300
  a = BodyBatch(bodies, g, dt, **kw)
  b = BodyBatch(bodies, g, dt, **kw)
  a.init()
  b.init()
  a.step(0)
  b.step(0)
  s = a.solver
  assert L.mgpbd_set_barrier_limit(s._h, 0.0) == 0
  s.make_prediction()
  x_before = a.x.clone()
  with pytest.raises(MGPBDError) as e:
    s.solve(1)
  assert e.value.code == ECUDA
  assert 'timed out' in str(e.value)
  st = C.c_uint32()
  N.check(L.mgpbd_get_status(s._h, C.byref(st)), 'mgpbd_get_status')
  assert st.value & SYNC_TIMEOUT
  torch.cuda.synchronize()
  assert L.mgpbd_set_barrier_limit(s._h, 4.0) == 0
  with torch.no_grad():
    a.x.copy_(x_before)
  s.solve(1)
  s.update_vel()
  b.step(1)
  assert s.stats()['status'] & SYNC_TIMEOUT == 0
  assert torch.isfinite(a.x).all()
  assert float((a.x - b.x).abs().max()) <= 1e-5 * float(b.x.abs().max())
