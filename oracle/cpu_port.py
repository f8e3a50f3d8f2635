"""ctypes wrapper of oracle/cpu_step.cpp, the OpenMP CPU port of the MGPBD
step (TEST / MEASUREMENT INFRASTRUCTURE: bench.py's CPU baseline and
`--impl reference` arm time it; the product never uses it).

The integer structure comes from the numpy oracle (its restatement of the
reference's pattern, aggregation and Galerkin setup); the first matrix for
the Galerkin zero-dropping is the float32 oracle's.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from . import mgpbd_oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'libcpu_step.so')
SRC = os.path.join(HERE, 'cpu_step.cpp')


def build(force=False):
  if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
    return LIB
  os.makedirs(BUILD, exist_ok=True)
  tmp = LIB + '.tmp'
  cmd = ['g++', '-std=c++17', '-O3', '-fopenmp', '-shared', '-fPIC', SRC, '-o', tmp]
  r = subprocess.run(cmd, capture_output=True, text=True)
  if r.returncode != 0:
    raise RuntimeError(f'CPU port build failed: {" ".join(cmd)}\n{r.stderr}')
  os.replace(tmp, LIB)
  return LIB


_lib = None


def lib():
  global _lib
  if _lib is None:
    L = C.CDLL(build())
    vp, i32, f32, f64 = C.c_void_p, C.c_int32, C.c_float, C.c_double
    L.cpu_create.restype = vp
    L.cpu_create.argtypes = [i32, i32, vp, vp, vp, vp, f32, f32, f32, f32, vp, i32, f64, f64, i32,
                             f64, f64, i32, f64, i32, vp]
    L.cpu_destroy.argtypes = [vp]
    L.cpu_add_level.argtypes = [vp, i32, vp, vp, C.c_int64, vp, vp, vp]
    L.cpu_predict.argtypes = [vp]
    L.cpu_update_vel.argtypes = [vp]
    L.cpu_newton_iteration.restype = C.c_int
    L.cpu_newton_iteration.argtypes = [vp, i32, C.POINTER(f64), i32, vp]
    L.cpu_get_x.argtypes = [vp, vp]
    L.cpu_threads.restype = C.c_int
    _lib = L
  return _lib


def _c(a, dt):
  return np.ascontiguousarray(a, dtype=dt)


class CpuPort:
  """The plain MGPBD step on the host cores (float32, OpenMP)."""

  def __init__(self, x0, x_ref, invm, t_i, gravity, dt, mu=1e6, compliance=0.0, damp=1.0,
               maxiter=20, atol=1e-4, rtol=1e-2, maxiter_cg=100, tol_cg=1e-5, rel_tol_cg=0.0,
               n_smooth=2, omega_jacobi=2.0 / 3.0, kinematic_pins=False, ctype=None,
               hierarchy=None):
    """ctype: per-constraint types (0 ARAP, 1 length (a, b, a, b), 2
    volume), None for all ARAP; hierarchy: level-0 aggregate ids to use
    instead of the tet aggregation."""
    L = lib()
    self.maxiter = maxiter
    self.maxiter_cg = maxiter_cg
    self._keep = [_c(x_ref, np.float32), _c(x0, np.float32), _c(invm, np.float32),
                  _c(t_i, np.int32), _c(gravity, np.float32)]
    xr, x, w, t, g = self._keep
    self.nv = len(xr)
    self.nt = len(t) // 4
    ct = None if ctype is None else _c(ctype, np.int32)
    self._keep.append(ct)
    self.h = L.cpu_create(self.nv, self.nt, xr.ctypes.data, x.ctypes.data, w.ctypes.data,
                          t.ctypes.data, dt, mu, compliance, damp, g.ctypes.data, maxiter, atol,
                          rtol, maxiter_cg, tol_cg, rel_tol_cg, n_smooth, omega_jacobi,
                          int(bool(kinematic_pins)), None if ct is None else ct.ctypes.data)
    self.compliance = float(compliance)
    self.n_mesh_tets = self.nt if ctype is None else int(np.sum(np.asarray(ctype) != 1))
    # structure from the oracle restatement
    ip, ix = orc.sparsity_pattern(t, self.nt)
    self.nnz0 = int(len(ix))
    L.cpu_add_level(self.h, self.nt, ip.ctypes.data, ix.ctypes.data, len(ix), None, None, None)
    if hierarchy is not None:
      aggs, sizes = [np.asarray(hierarchy)], [self.nt, int(np.max(hierarchy)) + 1]
    else:
      aggs, sizes = orc.tet_hierarchy(t, self.nt)
    if aggs:
      dm, rest, al = orc.rest_shape(xr, t, mu, dt, np.float32, compliance, ct)
      C0, g0 = orc.constraints(x, t, dm, np.float32, ct, rest)
      a0 = orc.fill_A(ip, ix, t, w, g0, al, np.float32)
      ci, cx, cidx, coff, _ = orc.galerkin(ip, ix, a0, aggs[0], sizes[1])
      agg = _c(aggs[0], np.int32)
      self._keep += [ip, ix, ci, cx, cidx, coff, agg]
      L.cpu_add_level(self.h, sizes[1], ci.ctypes.data, cx.ctypes.data, len(cx), agg.ctypes.data,
                      coff.ctypes.data, cidx.ctypes.data)
    else:
      self._keep += [ip, ix]
    self.log = []

  def __del__(self):
    if getattr(self, 'h', None):
      lib().cpu_destroy(self.h)
      self.h = None

  def newton_iteration(self, ite, r0, cg_max=None):
    out = np.zeros(8, np.float64)
    done = lib().cpu_newton_iteration(self.h, ite, C.byref(r0),
                                      self.maxiter_cg if cg_max is None else cg_max,
                                      out.ctypes.data)
    return bool(done), out

  def step(self):
    L = lib()
    L.cpu_predict(self.h)
    r0 = C.c_double(0.0)
    self.log = []
    for ite in range(self.maxiter):
      done, out = self.newton_iteration(ite, r0)
      self.log.append(out.copy())
      if done:
        break
    L.cpu_update_vel(self.h)

  def positions(self):
    x = np.empty((self.nv, 3), np.float32)
    lib().cpu_get_x(self.h, x.ctypes.data)
    return x


def threads():
  return lib().cpu_threads()
