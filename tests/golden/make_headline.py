"""Recipe of the headline-configuration fixtures (float64 oracle, exact
linear solves): run here on the CPU, the fixtures are committed.

    python tests/golden/make_headline.py c1            # -> headline_c1.npz
    python tests/golden/make_headline.py cube N S K [cheb]
                              # -> headline_N_seedS.npz (headline_N_seedS_cheb.npz)

* c1: the 10 x 10 x 10 hex cube (1,331 vertices, 5,000 tets; length +
  volume constraints), compliance 1e-6, 100 frames x 5 substeps (dt 1/300),
  top face pinned, jitter +-0.01 h from seed 0.  Positions after substeps
  1..20 and every 20th substep after that.
* cube: the N x N x N cube of the benchmark (N = 40: the benchmark's body)
  with the compliance that seed S draws (log-uniform in [1e-9, 1e-4]), K
  substeps; displacements from the start positions after each.  The 40^3
  runs solve K by CG (about 2 minutes per solve single-threaded); the
  stiffest draws run on 20^3, where K is factorised.

Newton settings are the benchmark's (maxiter 20, atol 1e-4, rtol 1e-2, no
damping, pinned vertices kinematic).  Each Newton system is solved to a
float64 dual residual of 1e-11 |b| (oracle/exact_solve.py), or, with
`cheb`, by the library's FAST linear solve restated in float64 (Chebyshev-8
CG on A to relative residual 1e-6): the same algorithm as the CUDA path.  The Newton log
of every substep (residual per iteration) is stored with the positions, so
a test can see how far each substep's Newton test was from its threshold.
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from controllable_pbd_3d_gb300 import meshgen  # noqa: E402
from oracle import mgpbd_oracle as MO  # noqa: E402

DT = 1.0 / 300.0
NEWTON = dict(damp=1.0, maxiter=20, atol=1e-4, rtol=1e-2, kinematic_pins=True)


def cube(n, seed):
  """The benchmark body: n^3 hexes (h = 1/n), jitter +-0.01 h from seed, top
  face pinned, compliance log-uniform in [1e-9, 1e-4] from the same seed."""
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.01, seed=seed)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  compliance = float(10.0 ** np.random.default_rng(seed).uniform(-9.0, -4.0))
  return xr, x0, t, invm, compliance


def run(n, seed, compliance, substeps, keep, linear='exact'):
  xr, x0, t, invm, drawn = cube(n, seed)
  comp = drawn if compliance is None else compliance
  c, ty, _, _ = MO.edge_volume_system(t)
  o = MO.MGPBDOracle(x0, xr, invm, c, [0.0, -9.8, 0.0], DT, dtype=np.float64, compliance=comp,
                     ctype=ty, linear=linear, rel_tol_cg=1e-6, tol_cg=1e-12, maxiter_cg=6000,
                     **NEWTON)
  o.init()
  snaps, idx, logs = [], [], []
  t0 = time.perf_counter()
  for i in range(substeps):
    o.step(i // 5)
    logs.append([r for (_, r, _, _) in o.log])
    if keep(i + 1):
      snaps.append(o.x.copy())
      idx.append(i + 1)
    print(f'substep {i + 1}: newton residuals {logs[-1]}, '
          f'{time.perf_counter() - t0:.1f} s', flush=True)
  width = max(len(l) for l in logs)
  res = np.full((substeps, width), np.nan)
  for i, l in enumerate(logs):
    res[i, :len(l)] = l
  return dict(x0=x0, snaps=np.array(snaps), substeps=np.array(idx), newton_residuals=res,
              compliance=comp, n=n, seed=seed)


def main():
  case = sys.argv[1]
  if case == 'c1':
    d = run(10, 0, 1e-6, 500, lambda k: k <= 20 or k % 20 == 0)
    np.savez_compressed(os.path.join(HERE, 'headline_c1.npz'), x=d['snaps'].astype(np.float32),
                        substeps=d['substeps'], newton_residuals=d['newton_residuals'],
                        compliance=d['compliance'])
  elif case == 'cube':
    n, seed, k = int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4])
    linear = sys.argv[5] if len(sys.argv) > 5 else 'exact'
    d = run(n, seed, None, k, lambda k: True, linear)
    disp = (d['snaps'] - d['x0'][None].astype(np.float64)).astype(np.float32)
    tag = '' if linear == 'exact' else f'_{linear}'
    np.savez_compressed(os.path.join(HERE, f'headline_{n}_seed{seed}{tag}.npz'), disp=disp,
                        substeps=d['substeps'], newton_residuals=d['newton_residuals'],
                        compliance=d['compliance'])
  else:
    raise SystemExit(__doc__)


if __name__ == '__main__':
  main()
