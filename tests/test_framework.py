"""The MGPBD step behind the pbd_framework constraint interface
(cons/framework.py:6-89): a framework-driven substep (its own prediction and
velocity update, one Newton iteration per update_cons) lands where
MGPBDSolverGPU.step lands."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('mode', ['parity', 'fast'])
def test_framework_adapter_matches_step(cuda, mode):
  from controllable_pbd_3d_gb300 import meshgen
  from controllable_pbd_3d_gb300.framework import MGPBDConstraint, PbdFramework
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  n = 6
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=11)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  kw = dict(mu=1e5, damp=1.0, maxiter=6, rtol=1e-6, atol=1e-9, maxiter_cg=400, tol_cg=1e-10,
            rel_tol_cg=1e-7, mode=mode)
  if mode == 'fast':
    kw['smoother'] = 'safe'
  g, dt = [0.0, -9.8, 0.0], 1 / 300

  def make(x):
    s = MGPBDSolverGPU(x, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                       cuda.tensor(t, device='cuda'), None, g, dt, **kw)
    return s

  xa = cuda.tensor(x0, device='cuda')
  sa = make(xa)
  sa.init()
  xb = cuda.tensor(x0, device='cuda')
  sb = make(xb)
  fw = PbdFramework(xb, g, dt, damp=1.0)
  con = MGPBDConstraint(sb)
  fw.add_cons(con)
  fw.init_rest_status()
  for k in range(3):
    sa.step(k)
    fw.step(subsub=kw['maxiter'])
    assert len(con.log) == len(sa.newton_log())
  scale = float(np.abs(x0).max())
  assert float((xa - xb).abs().max()) <= 1e-5 * scale
  assert float((sa.v_v - fw.v_v).abs().max()) <= 1e-3 * max(float(sa.v_v.abs().max()), 1e-6)
