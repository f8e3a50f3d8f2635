"""Row-kernel autotuner: the candidate shapes (CPU), every shape computing
the same sweep on a real level matrix, the tuner's choice, the JSON cache
round trip (GPU)."""

import ctypes as C
import json

import numpy as np
import pytest

from controllable_pbd_3d_gb300 import _native as N


def test_candidate_shapes():
  L = N.lib()
  n = C.c_int32()
  assert L.mgpbd_row_shapes(None, C.byref(n)) == 0
  codes = (C.c_int32 * n.value)()
  assert L.mgpbd_row_shapes(codes, C.byref(n)) == 0
  codes = list(codes)
  assert codes[0] == 406 and len(set(codes)) == len(codes) == 8
  for c in codes:
    g, u = divmod(c, 100)
    assert g in (2, 4, 8) and 4 * g * u <= 128


def plain_solver(torch, n=10):
  from controllable_pbd_3d_gb300 import meshgen
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  xr, t = meshgen.hex_grid_tets(n, n, n, h=1.0 / n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, h=1.0 / n, jitter=0.05, seed=1)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  s = MGPBDSolverGPU(torch.tensor(x0, device='cuda'), torch.tensor(xr, device='cuda'),
                     torch.tensor(invm, device='cuda'), torch.tensor(t, device='cuda'), None,
                     [0.0, -9.8, 0.0], 1.0 / 300, smoother='safe', kinematic_pins=True,
                     compliance=1.5e-6, maxiter=2, maxiter_cg=2000, rel_tol_cg=1e-6, tol_cg=0.0)
  s.init()
  s._compute_C_and_gradC()
  s._fill_A_and_update_gpu()
  return s


@pytest.mark.gpu
def test_every_shape_computes_the_same_sweep(cuda):
  torch = cuda
  s = plain_solver(torch)
  L = N.lib()
  n = C.c_int32()
  L.mgpbd_row_shapes(None, C.byref(n))
  codes = (C.c_int32 * n.value)()
  L.mgpbd_row_shapes(codes, C.byref(n))
  for level in range(s.stats()['n_levels']):
    rows = s.stats()['rows'][level]
    g = torch.Generator(device='cuda').manual_seed(level)
    x = torch.randn(rows, device='cuda', generator=g)
    b = torch.randn(rows, device='cuda', generator=g)
    ref_y = ref_j = None
    for c in list(codes):
      s.set_row_shape(level, c)
      assert s.row_shape(level) == c
      y = s.level_sweep(level, 0, x).cpu().numpy().astype(np.float64)
      j = s.level_sweep(level, 1, x, b, omega=0.6).cpu().numpy().astype(np.float64)
      if ref_y is None:
        ref_y, ref_j = y, j
      assert np.abs(y - ref_y).max() <= 1e-5 * np.abs(ref_y).max(), (level, c)
      assert np.abs(j - ref_j).max() <= 1e-5 * np.abs(ref_j).max(), (level, c)
    s.set_row_shape(level, 0)
    assert s.row_shape(level) == 0


@pytest.mark.gpu
def test_autotune_and_cache_round_trip(cuda, tmp_path):
  torch = cuda
  s = plain_solver(torch)
  cache = str(tmp_path / 'rows.json')
  got = s.autotune(reps=3, cache=cache)
  nl = s.stats()['n_levels']
  assert sorted(got) == list(range(nl))
  for l in range(nl):
    assert s.row_shape(l) == got[l] and got[l] > 0
    assert s.last_tuning[l][1] > 0.0
  table = json.load(open(cache))
  assert len(table) == nl
  # a second solver of the same shape takes the cached shapes without timing
  s2 = plain_solver(torch)
  s2.last_tuning = None
  assert s2.autotune(cache=cache) == got
  assert s2.last_tuning is None
  # a tuned solver still converges like the default one
  s2.step(0)
  assert s2.stats()['newton_iters'] == 2 and not (s2.stats()['status'] & 1)
