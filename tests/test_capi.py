"""The C-ABI library: it loads, exports every symbol include/mgpbd.h and
include/mgpbd_local.h declare, and its host-only entry points validate
arguments.  No GPU."""

import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from controllable_pbd_3d_gb300 import _native as N


def declared():
  names = set()
  for h in ('mgpbd.h', 'mgpbd_local.h'):
    hdr = open(os.path.join(ROOT, 'include', h)).read()
    names |= set(re.findall(r'\b(mgpbd_[a-z_0-9]+)\s*\(', hdr))
  return sorted(names)


def test_library_loads_and_exports_every_declared_symbol():
  L = N.lib()
  names = declared()
  assert len(names) >= 40
  for n in names:
    assert hasattr(L, n), n
  out = subprocess.run(['nm', '-D', '--defined-only', N.lib_path()], capture_output=True,
                       text=True).stdout
  exported = {ln.split()[-1] for ln in out.splitlines() if ' T mgpbd_' in ln}
  assert set(names) == exported


def test_ctypes_signatures_cover_the_header():
  assert set(N._SIGS) == set(declared())


def test_local_params_struct_layout():
  assert C.sizeof(N.XpbdParams) == 16
  assert C.sizeof(N.VbdParams) == 4 * 11


def test_params_struct_layout():
  p = N.default_params()
  # every field is 4 bytes; gravity counts 3
  assert C.sizeof(N.Params) == 4 * (len(N.Params._fields_) + 2)
  assert abs(p.mu - 1e6) < 1 and p.maxiter == 20 and p.maxiter_cg == 100
  assert abs(p.omega_jacobi - 2.0 / 3.0) < 1e-7 and p.use_line_search == 1
  assert p.mode == N.MGPBD_MODE_PARITY and p.cg_alias == 0
  assert p.body_cg == 1


def test_error_codes_and_strings():
  L = N.lib()
  assert L.mgpbd_strerror(0) == b'ok'
  assert L.mgpbd_strerror(-1) == b'invalid argument'
  assert L.mgpbd_create(None, None) == -1
  p = N.default_params()
  h = C.c_void_p()
  # dt must be positive
  assert L.mgpbd_create(C.byref(p), C.byref(h)) == -1
  assert b'dt' in L.mgpbd_last_error()
  # calls on a null handle
  assert L.mgpbd_init(None) == -1
  assert L.mgpbd_step(None, 0) == -1


def test_host_entry_points_validate():
  L = N.lib()
  nnz = C.c_int64()
  assert L.mgpbd_host_pattern(None, 1, C.byref(nnz), None, None) == -1
  t = np.array([0, 1, 2, 3], np.int32)
  agg = np.zeros(1, np.int32)
  n = C.c_int32()
  assert L.mgpbd_host_aggregate(t.ctypes.data, 1, 0, agg.ctypes.data, C.byref(n)) == -1
  assert L.mgpbd_host_aggregate(t.ctypes.data, 1, 8, agg.ctypes.data, C.byref(n)) == 0
  assert n.value == 1


def test_step_before_init_is_a_state_error():
  pytest.importorskip('torch')
  L = N.lib()
  p = N.default_params()
  p.dt = 1.0 / 300
  h = C.c_void_p()
  assert L.mgpbd_create(C.byref(p), C.byref(h)) == 0
  try:
    assert L.mgpbd_step(h, 0) == -4
    assert L.mgpbd_init(h) == -4  # no mesh bound
  finally:
    L.mgpbd_destroy(h)


def test_stats_struct_layout_matches_the_header(tmp_path):
  """ctypes' mgpbd_stats has the C compiler's size and field offsets."""
  src = tmp_path / 'lay.c'
  fields = [f for f, _ in N.Stats._fields_]
  body = '\n'.join(f'  printf("%s %zu\\n", "{f}", offsetof(mgpbd_stats, {f}));' for f in fields)
  src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "mgpbd.h"\nint main(void) {\n'
                 f'  printf("size %zu\\n", sizeof(mgpbd_stats));\n{body}\n  return 0;\n}}\n')
  exe = tmp_path / 'lay'
  subprocess.run(['gcc', '-I', os.path.join(ROOT, 'include'), str(src), '-o', str(exe)], check=True)
  out = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True,
                                                  check=True).stdout.splitlines())
  assert int(out['size']) == C.sizeof(N.Stats)
  for f in fields:
    assert int(out[f]) == getattr(N.Stats, f).offset, f


def test_dot_noalloc_rejects_bad_sizes_with_a_message():
  """The allocation-free dot product checks its size against the fixed
  scratch before any CUDA call and leaves a message (no GPU needed)."""
  import ctypes as C
  L = N.lib()
  out = C.c_double(-1.0)
  assert L.mgpbd_dot_noalloc(67_108_864 + 1, C.c_void_p(16), C.c_void_p(16), C.byref(out),
                             None) == -6  # MGPBD_ERANGE
  assert b'67,108,864' in L.mgpbd_last_error()
  assert L.mgpbd_dot_noalloc(-1, None, None, C.byref(out), None) == -1  # MGPBD_EINVAL
  assert b'mgpbd_dot_noalloc' in L.mgpbd_last_error()


def test_integration_stub_mirrors_the_params_struct():
  """The ctypes stub a maintainer would copy
  lists the fields of mgpbd_params in the header's order, as the binding
  does."""
  import os
  import re
  here = os.path.dirname(os.path.abspath(__file__))
  text = open(os.path.join(here, '..', 'INTEGRATION.md')).read()
  block = text[text.index('class Params(C.Structure)'):]
  block = block[:block.index(']\n') + 1]
  names = re.findall(r"\('([a-z_0-9]+)',", block)
  assert names == [f[0] for f in N.Params._fields_]
  header = open(os.path.join(here, '..', 'include', 'mgpbd.h')).read()
  struct = header[header.index('typedef struct mgpbd_params {'):header.index('} mgpbd_params;')]
  fields = re.findall(r'^\s+(?:float|int32_t)\s+([a-z_0-9]+)(?:\[3\])?;', struct, re.M)
  assert fields == names
