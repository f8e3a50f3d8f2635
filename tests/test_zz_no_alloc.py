"""mgpbd_dot_noalloc: the dot product for callers that may not allocate GPU
memory (hosts that own the device memory budget forbid cudaMalloc inside
the library, since it can wait for the whole device).  Its result must equal
mgpbd_dot's, call after call, although both share one fixed scratch array.

Kept in its own file, named to be collected last.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dot(L, fn, a, b, stream):
  out = C.c_double()
  rc = getattr(L, fn)(a.numel(), a.data_ptr(), b.data_ptr(), C.byref(out), C.c_void_p(stream))
  assert rc == 0, (fn, rc)
  return out.value


@pytest.mark.parametrize('n', [1, 1000, 123457, 3_000_001])
def test_dot_noalloc_matches_dot_twice(cuda, n):
  from controllable_pbd_3d_gb300 import _native as N
  torch = cuda
  L = N.lib()
  g = torch.Generator(device='cuda').manual_seed(n)
  stream = torch.cuda.current_stream().cuda_stream
  for call in range(2):
    a = torch.randn(n, device='cuda', generator=g)
    b = torch.randn(n, device='cuda', generator=g)
    ref = _dot(L, 'mgpbd_dot', a, b, stream)
    got = _dot(L, 'mgpbd_dot_noalloc', a, b, stream)
    exact = float(np.dot(a.cpu().numpy().astype(np.float64), b.cpu().numpy().astype(np.float64)))
    scale = float(np.sum(np.abs(a.cpu().numpy().astype(np.float64) * b.cpu().numpy())))
    assert abs(got - ref) <= 1e-12 * max(scale, 1e-30), (call, got, ref)
    assert abs(got - exact) <= 1e-12 * max(scale, 1e-30), (call, got, exact)


def test_dot_noalloc_empty_and_limit(cuda):
  from controllable_pbd_3d_gb300 import _native as N
  torch = cuda
  L = N.lib()
  stream = torch.cuda.current_stream().cuda_stream
  a = torch.ones(10, device='cuda')
  assert _dot(L, 'mgpbd_dot_noalloc', a, a, stream) == 10.0
  out = C.c_double(-1.0)
  # n = 0 gives 0, not the previous call's result
  assert L.mgpbd_dot_noalloc(0, None, None, C.byref(out), C.c_void_p(stream)) == 0
  assert out.value == 0.0
  # beyond the scratch limit: a clear range error, nothing launched
  too_many = 67_108_864 + 1
  assert L.mgpbd_dot_noalloc(too_many, a.data_ptr(), a.data_ptr(), C.byref(out),
                             C.c_void_p(stream)) == -6
  assert L.mgpbd_strerror(-6) == b'size out of range'
  assert b'67,108,864' in L.mgpbd_last_error()
  assert L.mgpbd_dot_noalloc(-1, None, None, C.byref(out), C.c_void_p(stream)) == -1
  assert b'mgpbd_dot_noalloc' in L.mgpbd_last_error()
