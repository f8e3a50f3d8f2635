"""The OpenMP CPU port (bench's CPU baseline) agrees with the float64 oracle."""

import numpy as np
import pytest

from controllable_pbd_3d_gb300 import meshgen


@pytest.mark.parametrize('kinematic', [False, True])
def test_cpu_port_matches_float64_oracle(kinematic):
  from oracle.cpu_port import CpuPort
  from oracle.mgpbd_oracle import MGPBDOracle
  n = 8
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=3)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  kw = dict(mu=1e5, damp=0.993, maxiter=5, rtol=1e-6, atol=1e-9, maxiter_cg=400, tol_cg=1e-12,
            rel_tol_cg=1e-7, kinematic_pins=kinematic)
  o = MGPBDOracle(x0, xr, invm, t, [0, -9.8, 0], 1 / 300, dtype=np.float64, smoother='safe', **kw)
  o.init()
  p = CpuPort(x0, xr, invm, t, [0, -9.8, 0], 1 / 300, **kw)
  for k in range(2):
    o.step(k)
    p.step()
  err = float(np.abs(p.positions() - o.x).max())
  assert err <= 1e-5 * float(np.abs(o.x).max()), err
