"""A numpy stand-in for the parts of the Taichi runtime the MGPBD step uses.

Purpose: run the reference's own `cons/*.py` solver code, unmodified, on the
CPU of this container (Taichi itself is not installed) so that its outputs
can be stored as golden fixtures.  Installing this module as `taichi` in
`sys.modules` turns every `@ti.kernel` into a plain serial Python loop:

* fields are numpy arrays (float32 / int32), vector and matrix fields keep
  their element as trailing axes, and indexing a vector/matrix field returns a
  *view*, so `ti.atomic_add(field[i], v)` and `field[i] += v` update storage;
* scalar arithmetic stays float32 (numpy's weak Python-scalar promotion);
* kernel return values become Python floats, as Taichi returns them;
* vector / matrix methods (`dot`, `norm_sqr`, `normalized`, `cross`, `outer_product`,
  `inverse`, `determinant`, `Matrix.identity`) as float32 numpy operations
  (inverse and determinant through float64 LAPACK);
* `ti.svd` is the rotation-variant SVD (U, V proper rotations, the sign of
  det F carried by the last singular value), computed in float64 from
  LAPACK and rounded to float32.

What this cannot reproduce: Taichi's own f32 SVD iteration and the order of
its parallel f32 atomic reductions.  Fixtures made with it pin the reference's
control flow, index structures and operation order, not those two.
"""

from __future__ import annotations

import sys
import types
from functools import wraps

import numpy as np

f32 = np.float32
f64 = np.float64
i32 = np.int32


class TiArray(np.ndarray):
  """numpy array with the few Taichi field/vector/matrix methods used."""

  # field API
  def from_numpy(self, a):
    self[...] = np.asarray(a).reshape(self.shape)

  def to_numpy(self):
    return np.array(self).view(np.ndarray).copy()

  # vector API
  def dot(self, o):
    return np.add.reduce(np.asarray(self) * np.asarray(o))

  def norm_sqr(self):
    # sum of squares of every entry, in row-major order (vectors and
    # matrices alike)
    a = np.asarray(self).reshape(-1)
    acc = a.dtype.type(0)
    for v in a:
      acc = acc + v * v
    return acc

  def cross(self, o):
    a, b = np.asarray(self), np.asarray(o)
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]], dtype=a.dtype).view(TiArray)

  def outer_product(self, o):
    return np.outer(np.asarray(self), np.asarray(o)).view(TiArray)

  @property
  def n(self):
    return self.shape[-1]

  def norm(self):
    return np.sqrt(self.norm_sqr())

  def normalized(self):
    # the vector over its norm, in the element type
    return (np.asarray(self) / self.norm()).view(TiArray)

  # matrix API
  def inverse(self):
    return np.linalg.inv(np.asarray(self, np.float64)).astype(self.dtype).view(TiArray)

  def determinant(self):
    return self.dtype.type(np.linalg.det(np.asarray(self, np.float64)))


class _Scalar0D:
  """0-d field, indexed with `[None]`."""

  def __init__(self, dtype):
    self.a = np.zeros((), dtype)

  def __getitem__(self, key):
    return self.a[()]

  def __setitem__(self, key, val):
    self.a[()] = val

  def fill(self, v):
    self.a[()] = v

  def to_numpy(self):
    return self.a.copy()


def _shape(shape):
  if isinstance(shape, (int, np.integer)):
    return (int(shape),)
  return tuple(int(s) for s in shape)


def field(dtype=f32, shape=()):
  shape = _shape(shape)
  if shape == ():
    return _Scalar0D(dtype)
  return np.zeros(shape, dtype).view(TiArray)


def _is_int(v):
  return isinstance(v, (int, np.integer)) and not isinstance(v, bool)


class Vector:
  """`ti.Vector([...])` constructor plus `ti.Vector.field`."""

  def __new__(cls, vals, dt=None):
    vals = list(vals)
    if dt is None:
      dt = i32 if all(_is_int(v) for v in vals) else f32
    return np.array(vals, dtype=dt).view(TiArray)

  @staticmethod
  def field(n, dtype=f32, shape=()):
    return np.zeros(_shape(shape) + (n,), dtype).view(TiArray)


class Matrix:

  def __new__(cls, rows, dt=None):
    return np.array(rows, dtype=dt or f32).view(TiArray)

  @staticmethod
  def field(n, m, dtype=f32, shape=()):
    return np.zeros(_shape(shape) + (n, m), dtype).view(TiArray)

  @staticmethod
  def cols(cols):
    return np.stack([np.asarray(c) for c in cols], axis=1).view(TiArray)

  @staticmethod
  def identity(dt=f32, n=3):
    return np.eye(n, dtype=dt).view(TiArray)


MatrixField = TiArray
Field = TiArray


def svd(F):
  """Rotation-variant SVD: F = U diag(s) V^T with det U = det V = +1."""
  A = np.asarray(F, np.float64)
  u, s, vt = np.linalg.svd(A)
  v = vt.T.copy()
  s = s.copy()
  if np.linalg.det(u) < 0:
    u[:, 2] *= -1.0
    s[2] *= -1.0
  if np.linalg.det(v) < 0:
    v[:, 2] *= -1.0
    s[2] *= -1.0
  dt = np.asarray(F).dtype
  return (u.astype(dt).view(TiArray), np.diag(s).astype(dt).view(TiArray),
          v.astype(dt).view(TiArray))


def sqrt(x):
  return np.sqrt(x)


def abs(x):  # noqa: A001 - Taichi name
  return np.abs(x)


def atomic_add(ref, val):
  old = np.array(ref, copy=True)
  ref += val
  return old


def static(x):
  return x


def kernel(fn):
  @wraps(fn)
  def run(*args, **kwargs):
    r = fn(*args, **kwargs)
    if isinstance(r, np.floating):
      return float(r)
    return r
  return run


def func(fn):
  return fn


def data_oriented(cls):
  return cls


def template():
  return None


def loop_config(**kwargs):
  return None


def init(*args, **kwargs):
  return None


def sync():
  return None


class _Types:

  @staticmethod
  def ndarray(dtype=None, ndim=None):
    return None


types_ns = _Types()


def install():
  """Register this module as `taichi` (and `taichi.math`) in sys.modules."""
  mod = sys.modules[__name__]
  ti = types.ModuleType('taichi')
  for name in ('f32', 'f64', 'i32', 'field', 'Vector', 'Matrix', 'MatrixField',
               'Field', 'svd', 'sqrt', 'abs', 'atomic_add', 'static', 'kernel',
               'func', 'data_oriented', 'template', 'loop_config', 'init', 'sync'):
    setattr(ti, name, getattr(mod, name))
  ti.types = types_ns
  ti.math = types.SimpleNamespace(vec3=None)
  ti.x64 = 'x64'
  ti.cpu = 'cpu'
  ti.cuda = 'cuda'
  ti.vulkan = 'vulkan'
  sys.modules['taichi'] = ti
  return ti
