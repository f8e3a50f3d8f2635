"""`SolverBenchmark` keeps the reference recorder's API and JSON layout
(`utils/bench.py:14-97`): a record the reference wrote
(`tests/golden/solver_benchmark_ref.json`, made by
`tests/golden/make_bench_record.py`) loads, summarises to the reference's
own summary, and saves back to the same text; a record made here has the
same keys.  Host only."""

import json
import os

import pytest

from conftest import GOLDEN

from controllable_pbd_3d_gb300.solver_benchmark import SolverBenchmark


def _read(name):
  with open(os.path.join(GOLDEN, name)) as f:
    return f.read()


def test_reference_record_loads_summarises_and_saves_unchanged(tmp_path):
  b = SolverBenchmark.load(os.path.join(GOLDEN, 'solver_benchmark_ref.json'))
  ref_summary = json.loads(_read('solver_benchmark_ref_summary.json'))
  got = b.summary()
  assert set(got) == set(ref_summary)
  for k, v in ref_summary.items():
    if isinstance(v, float):
      assert got[k] == pytest.approx(v, rel=0, abs=0)
    else:
      assert got[k] == v
  out = tmp_path / 'again.json'
  b.save(str(out))
  assert out.read_text() == _read('solver_benchmark_ref.json')


def test_new_record_has_the_reference_layout(tmp_path):
  ref = json.loads(_read('solver_benchmark_ref.json'))
  b = SolverBenchmark('mgpbd', 'cube_10', {'dt': 1.0 / 300})
  b.record_iteration(0, 1.0)  # outside a frame: ignored, as in the reference
  b.end_frame()
  assert b.frames == []
  b.begin_frame(0)
  b.record_iteration(0, 0.5, cg_iters=12, omega=0.9)
  b.record_iteration(1, 0.25, cg_iters=30, omega=0.9, t=123.0)  # a library timestamp
  b.end_frame()
  path = tmp_path / 'rec.json'
  b.save(str(path))
  data = json.loads(path.read_text())
  assert list(data) == list(ref)
  fr, rf = data['frames'][0], ref['frames'][0]
  assert list(fr) == list(rf)
  assert list(fr['iterations'][0]) == list(rf['iterations'][0])
  assert fr['iterations'][1]['t'] == 123.0
  # frames read like the reference recorder's dicts
  f0 = b.frames[0]
  assert f0['frame_id'] == 0 and f0['iterations'][0]['cg_iters'] == 12
  with pytest.raises(KeyError):
    f0['nope']
  assert fr['t_start'] <= fr['iterations'][0]['t'] <= fr['t_end']
  s = SolverBenchmark.load(str(path)).summary()
  assert s['n_frames'] == 1 and s['avg_iterations'] == 2.0 and s['avg_final_residual'] == 0.25
  assert SolverBenchmark('a', 'b').summary() == {}


@pytest.mark.gpu
def test_solver_records_every_newton_iteration(cuda, tmp_path):
  """`MGPBDSolverGPU(..., benchmark=rec)` records one frame per solve and
  one entry per Newton iteration, with the library's residuals and CG
  counts, timestamps inside the frame."""
  torch = cuda
  from controllable_pbd_3d_gb300 import meshgen
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  x0, t, invm = meshgen.cube_body(6, jitter=0.02, seed=1)
  xr, _ = meshgen.hex_grid_tets(6, 6, 6)
  rec = SolverBenchmark('mgpbd', 'cube_6', {'mu': 1e5})
  x = torch.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], 1 / 300, mu=1e5,
                     benchmark=rec, maxiter=5)
  s.init()
  for f in range(2):
    s.step(f)
    st = s.stats()
    fr = rec.frames[-1]
    assert fr['frame_id'] == f
    # one entry per Newton solve, plus one without CG iterations when the
    # residual test ends the loop (cons/mgpbd_gpu.py:414-417)
    its = fr['iterations']
    assert len(its) in (st['newton_iters'], st['newton_iters'] + 1)
    if len(its) > st['newton_iters']:
      assert its[-1]['cg_iters'] == 0
    assert [it['iteration'] for it in its] == list(range(len(its)))
    assert sum(it['cg_iters'] for it in fr['iterations']) == st['cg_iters_total']
    assert all(it['residual'] >= 0 for it in fr['iterations'])
    assert all(fr['t_start'] <= it['t'] <= fr['t_end'] for it in fr['iterations'])
  assert len(rec.frames) == 2
  rec.save(str(tmp_path / 'r.json'))
  assert SolverBenchmark.load(str(tmp_path / 'r.json')).summary()['n_frames'] == 2
