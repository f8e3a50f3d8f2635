"""Convergence records of MGPBD substeps in the reference's JSON layout.

A record is a list of typed frame records (`FrameRecord`), each holding the
Newton iterations of one solve (`IterationRecord`: residual, CG iterations,
line-search step, timestamp).  `SolverBenchmark` is the recorder a solver
writes to (`MGPBDSolverGPU(..., benchmark=rec)` calls `begin_frame`,
`record_iteration` and `end_frame` around every solve); `write_record` /
`read_record` are the only places that know the file layout.

The layout is the one the reference's recorder writes (`utils/bench.py:
14-97`, class `SolverBenchmark`): top-level keys `solver_name`, `mesh_name`,
`params`, `frames`; per frame `frame_id`, `iterations`, `t_start`, `t_end`;
per iteration `iteration`, `residual`, `cg_iters`, `omega`, `t`; two-space
indented JSON.  The method names and the summary's keys are the reference
recorder's too, so its experiment and plotting scripts read these records
and call this recorder unchanged.

Timestamps use the host's monotonic clock (`time.perf_counter`).  The Newton
loop runs inside libmgpbd.so, which stamps each iteration with the same
clock at the synchronisation its residual test already makes; frame
boundaries synchronise the CUDA device first so a frame's time covers its
GPU work.
"""

from __future__ import annotations

import json
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

_FILE_KEYS = ('solver_name', 'mesh_name', 'params', 'frames')
_FRAME_KEYS = ('frame_id', 'iterations', 't_start', 't_end')
_ITER_KEYS = ('iteration', 'residual', 'cg_iters', 'omega', 't')


def _device_sync():
  try:
    import torch
  except ImportError:  # pragma: no cover
    return
  if torch.cuda.is_available():
    torch.cuda.synchronize()


@dataclass
class IterationRecord:
  """One Newton iteration: its dual residual norm, the CG iterations of its
  linear solve, the line-search step and when it finished."""
  iteration: int
  residual: float
  cg_iters: int
  omega: float
  t: float

  def as_layout(self) -> dict:
    return {'iteration': self.iteration, 'residual': self.residual, 'cg_iters': self.cg_iters,
            'omega': self.omega, 't': self.t}

  def __getitem__(self, key):
    """Read access by the layout's key, as code written against the
    reference recorder's dicts does (`it['residual']`)."""
    if key not in _ITER_KEYS:
      raise KeyError(key)
    return getattr(self, key)

  @classmethod
  def from_layout(cls, d: dict) -> 'IterationRecord':
    return cls(int(d['iteration']), float(d['residual']), int(d['cg_iters']), float(d['omega']),
               float(d['t']))


@dataclass
class FrameRecord:
  """One solve (frame or substep): its Newton iterations and its wall
  interval; t_end is None while the frame is open."""
  frame_id: int
  t_start: Optional[float]
  iterations: list = field(default_factory=list)
  t_end: Optional[float] = None

  @property
  def seconds(self) -> Optional[float]:
    if self.t_start is None or self.t_end is None:
      return None
    return self.t_end - self.t_start

  @property
  def final_residual(self) -> Optional[float]:
    return self.iterations[-1].residual if self.iterations else None

  def as_layout(self) -> dict:
    return {'frame_id': self.frame_id, 'iterations': [it.as_layout() for it in self.iterations],
            't_start': self.t_start, 't_end': self.t_end}

  def __getitem__(self, key):
    """Read access by the layout's key (`frame['iterations']`), as on the
    reference recorder's frame dicts."""
    if key not in _FRAME_KEYS:
      raise KeyError(key)
    return getattr(self, key)

  @classmethod
  def from_layout(cls, d: dict) -> 'FrameRecord':
    return cls(d['frame_id'], d['t_start'],
               [IterationRecord.from_layout(it) for it in d['iterations']], d['t_end'])


def write_record(path: str, solver_name: str, mesh_name: str, params: dict, frames) -> None:
  """Write frames in the reference's file layout."""
  doc = dict(zip(_FILE_KEYS, (solver_name, mesh_name, params,
                              [fr.as_layout() for fr in frames])))
  with open(path, 'w') as f:
    json.dump(doc, f, indent=2)


def read_record(path: str):
  """(solver_name, mesh_name, params, frames) of a record file."""
  with open(path) as f:
    doc = json.load(f)
  frames = [FrameRecord.from_layout(d) for d in doc['frames']]
  return doc['solver_name'], doc['mesh_name'], doc.get('params', {}), frames


def summarise(solver_name: str, mesh_name: str, frames) -> dict:
  """Mean / total frame time, mean Newton iterations and mean final
  residual over the frames (the reference summary's keys); {} when there
  are no frames."""
  if not frames:
    return {}
  secs = [s for s in (fr.seconds for fr in frames) if s is not None]
  counts = [len(fr.iterations) for fr in frames]
  finals = [r for r in (fr.final_residual for fr in frames) if r is not None]

  def mean(v):
    return float(np.mean(v)) if v else 0.0

  return {'solver_name': solver_name, 'mesh_name': mesh_name, 'n_frames': len(frames),
          'avg_frame_time': mean(secs), 'avg_iterations': mean(counts),
          'avg_final_residual': mean(finals),
          'total_time': float(np.sum(secs)) if secs else 0.0}


class SolverBenchmark:
  """Recorder of a solver's frames and Newton iterations (the reference
  recorder's interface).  Iterations recorded outside begin_frame /
  end_frame are dropped."""

  def __init__(self, solver_name: str, mesh_name: str, params: dict = None):
    self.solver_name = solver_name
    self.mesh_name = mesh_name
    self.params = params or {}
    self.frames: list = []
    self._open: Optional[FrameRecord] = None

  def begin_frame(self, frame_id: int):
    _device_sync()
    self._open = FrameRecord(frame_id, time.perf_counter())

  def record_iteration(self, iteration: int, residual: float, cg_iters: int = 0,
                       omega: float = 1.0, t: float | None = None):
    """t: the iteration's timestamp on the perf_counter clock (now if None)."""
    if self._open is None:
      return
    stamp = time.perf_counter() if t is None else t
    self._open.iterations.append(
        IterationRecord(int(iteration), float(residual), int(cg_iters), float(omega),
                        float(stamp)))

  def end_frame(self):
    if self._open is None:
      return
    _device_sync()
    self._open.t_end = time.perf_counter()
    self.frames.append(self._open)
    self._open = None

  def save(self, path: str):
    write_record(path, self.solver_name, self.mesh_name, self.params, self.frames)

  @staticmethod
  def load(path: str) -> 'SolverBenchmark':
    name, mesh, params, frames = read_record(path)
    rec = SolverBenchmark(name, mesh, params)
    rec.frames = frames
    return rec

  def summary(self) -> dict:
    return summarise(self.solver_name, self.mesh_name, self.frames)
