"""Writes tests/golden/geom3d_ref.npz: the reference's own lumped vertex
masses, tet volumes and face reversal (`utils/geom3d.py`, numpy only, imported
from the reference checkout) on a seeded jittered hex body.

    python tests/golden/make_geom_fixture.py <reference checkout>   (or REFERENCE_ROOT=<checkout>)
"""

import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from controllable_pbd_3d_gb300 import meshgen  # noqa: E402
from test_tet_data import boundary_triangles  # noqa: E402


def main(ref_root):
  spec = importlib.util.spec_from_file_location('ref_geom3d',
                                                os.path.join(ref_root, 'utils', 'geom3d.py'))
  geom = importlib.util.module_from_spec(spec)
  spec.loader.exec_module(geom)
  x, t = meshgen.hex_grid_tets(4, 3, 5, jitter=0.1, seed=3)
  x = x.astype(np.float64) * 1.7
  order, vm, tm = geom.compute_vertex_mass(x, t.astype(np.int64))
  f = boundary_triangles(t)
  rf = geom.revert_all_faces(f.copy())
  np.savez_compressed(os.path.join(HERE, 'geom3d_ref.npz'), x=x, t=t, order=order, vm=vm, tm=tm,
                      faces=f, reverted=rf)


if __name__ == '__main__':
  ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('REFERENCE_ROOT')
  if not ref:
    raise SystemExit(f'usage: python {sys.argv[0]} <reference checkout> (or set REFERENCE_ROOT)')
  main(ref)
