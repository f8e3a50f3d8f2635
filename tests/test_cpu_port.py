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


def test_cpu_port_edge_volume_matches_float64_oracle():
  """The same on the length + volume constraint system (the benchmark's
  construction)."""
  from controllable_pbd_3d_gb300.edge_volume import edge_volume_hierarchy, edge_volume_system
  from oracle.cpu_port import CpuPort
  from oracle.mgpbd_oracle import MGPBDOracle
  n = 6
  xr, t = meshgen.hex_grid_tets(n, n, n, h=1.0 / n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, h=1.0 / n, jitter=0.03, seed=2)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  c, types, _, _ = edge_volume_system(t)
  agg = edge_volume_hierarchy(t)
  kw = dict(damp=0.993, maxiter=5, rtol=1e-6, atol=1e-9, maxiter_cg=2000, tol_cg=1e-12,
            rel_tol_cg=1e-7, kinematic_pins=True, compliance=1e-6)
  o = MGPBDOracle(x0, xr, invm, c, [0, -9.8, 0], 1 / 300, dtype=np.float64, smoother='safe',
                  ctype=types, hierarchy=([agg], [len(types), int(agg.max()) + 1]), **kw)
  o.init()
  p = CpuPort(x0, xr, invm, c, [0, -9.8, 0], 1 / 300, ctype=types, hierarchy=agg, **kw)
  for k in range(2):
    o.step(k)
    p.step()
  err = float(np.abs(p.positions() - o.x).max())
  assert err <= 1e-5 * float(np.abs(o.x).max()), err
