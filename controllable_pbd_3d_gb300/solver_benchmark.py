"""Per-frame / per-iteration recorder with the API and JSON format of the
reference's `utils/bench.py:14-97` (`SolverBenchmark`).

Differences: the solver's Newton loop runs inside libmgpbd.so, so the
per-iteration timestamps come from the library's host clock (the same
monotonic clock as `time.perf_counter`), taken at the synchronisation the
loop already makes for its residual test; frame boundaries synchronise the
CUDA device instead of calling `ti.sync()`.
"""

from __future__ import annotations

import json
import time

import numpy as np


def _sync():
  try:
    import torch
    if torch.cuda.is_available():
      torch.cuda.synchronize()
  except ImportError:  # pragma: no cover
    pass


class SolverBenchmark:
  """Records per-frame, per-iteration timing and convergence data."""

  def __init__(self, solver_name: str, mesh_name: str, params: dict = None):
    self.solver_name = solver_name
    self.mesh_name = mesh_name
    self.params = params or {}
    self.frames = []
    self._current_frame = None

  def begin_frame(self, frame_id: int):
    _sync()
    self._current_frame = {'frame_id': frame_id, 'iterations': [], 't_start': time.perf_counter(),
                           't_end': None}

  def record_iteration(self, iteration: int, residual: float, cg_iters: int = 0,
                       omega: float = 1.0, t: float | None = None):
    if self._current_frame is None:
      return
    self._current_frame['iterations'].append({
        'iteration': int(iteration), 'residual': float(residual), 'cg_iters': int(cg_iters),
        'omega': float(omega), 't': float(t) if t is not None else time.perf_counter(),
    })

  def end_frame(self):
    if self._current_frame is None:
      return
    _sync()
    self._current_frame['t_end'] = time.perf_counter()
    self.frames.append(self._current_frame)
    self._current_frame = None

  def save(self, path: str):
    data = {'solver_name': self.solver_name, 'mesh_name': self.mesh_name, 'params': self.params,
            'frames': self.frames}
    with open(path, 'w') as f:
      json.dump(data, f, indent=2)

  @staticmethod
  def load(path: str) -> 'SolverBenchmark':
    with open(path) as f:
      data = json.load(f)
    b = SolverBenchmark(data['solver_name'], data['mesh_name'], data.get('params', {}))
    b.frames = data['frames']
    return b

  def summary(self) -> dict:
    if not self.frames:
      return {}
    frame_times, iters, final = [], [], []
    for fr in self.frames:
      if fr['t_end'] is not None and fr['t_start'] is not None:
        frame_times.append(fr['t_end'] - fr['t_start'])
      its = fr['iterations']
      iters.append(len(its))
      if its:
        final.append(its[-1]['residual'])
    return {
        'solver_name': self.solver_name, 'mesh_name': self.mesh_name, 'n_frames': len(self.frames),
        'avg_frame_time': float(np.mean(frame_times)) if frame_times else 0.0,
        'avg_iterations': float(np.mean(iters)) if iters else 0.0,
        'avg_final_residual': float(np.mean(final)) if final else 0.0,
        'total_time': float(np.sum(frame_times)) if frame_times else 0.0,
    }
