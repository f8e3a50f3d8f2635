"""Writes tests/golden/solver_benchmark_ref.json and
solver_benchmark_ref_summary.json with the reference's own recorder
(`utils/bench.py`, SolverBenchmark), imported from the reference checkout.
The timestamps are overwritten with fixed values so the files are stable.

    python tests/golden/make_bench_record.py <reference checkout>   (or REFERENCE_ROOT=<checkout>)
"""

import importlib.util
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
  spec = importlib.util.spec_from_file_location('ref_bench', os.path.join(ref_root, 'utils',
                                                                           'bench.py'))
  mod = importlib.util.module_from_spec(spec)
  spec.loader.exec_module(mod)
  b = mod.SolverBenchmark('mgpbd', 'cube_10', {'dt': 1.0 / 300, 'maxiter': 20, 'mu': 1e6})
  t = 100.0
  for f in range(3):
    b.begin_frame(f)
    b._current_frame['t_start'] = t
    for k in range(2 + f):
      b.record_iteration(k, 10.0 ** (-k - f), cg_iters=37 * (k + 1), omega=1.0 - 0.1 * k)
      b._current_frame['iterations'][-1]['t'] = t + 0.01 * (k + 1)
    b.end_frame()
    b.frames[-1]['t_end'] = t + 0.05 * (f + 1)
    t += 1.0
  b.begin_frame(3)  # an empty frame
  b._current_frame['t_start'] = t
  b.end_frame()
  b.frames[-1]['t_end'] = t + 0.02
  b.save(os.path.join(HERE, 'solver_benchmark_ref.json'))
  with open(os.path.join(HERE, 'solver_benchmark_ref_summary.json'), 'w') as f:
    json.dump(b.summary(), f, indent=2)


if __name__ == '__main__':
  ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('REFERENCE_ROOT')
  if not ref:
    raise SystemExit(f'usage: python {sys.argv[0]} <reference checkout> (or set REFERENCE_ROOT)')
  main(ref)
