"""ctypes binding of libmgpbd.so (the C ABI declared in include/mgpbd.h and
include/mgpbd_local.h).

The library is built in-tree by `controllable_pbd_3d_gb300.build`.  Loading
never falls back to another implementation: if the library is missing or a
symbol is absent, `lib()` raises.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

i32 = C.c_int32
i64 = C.c_int64
f32 = C.c_float
f64 = C.c_double
vp = C.c_void_p
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_f64 = C.POINTER(C.c_double)
P_u32 = C.POINTER(C.c_uint32)

MGPBD_MODE_PARITY = 0
MGPBD_MODE_FAST = 1
MGPBD_COARSE_JACOBI = 0
MGPBD_COARSE_DENSE_F64 = 1
MGPBD_SMOOTH_JACOBI = 0
MGPBD_SMOOTH_JACOBI_SAFE = 1
MGPBD_PRECOND_VCYCLE = 0
MGPBD_PRECOND_CHEB = 1
MGPBD_PRECOND_LEARNED = 2
MGPBD_CONS_ARAP = 0
MGPBD_CONS_LENGTH = 1
MGPBD_CONS_VOLUME = 2
MGPBD_NET_PARAMS = 16769
MGPBD_NET_LOSS_WEIGHTS = 0
MGPBD_NET_LOSS_FIELD = 1

STATUS_NAN = 1
STATUS_PAP_NONPOS = 2
STATUS_CG_MAXITER = 4
STATUS_NEWTON_MAXITER = 8
STATUS_STALL = 16

FIELD = {
    'lambdaf': 0, 'constraints': 1, 'gradC': 2, 'alpha_tilde': 3, 'rest_vol': 4,
    'Dm_inv': 5, 'v_p_old': 6, 'v_predict': 7, 'dpos': 8, 'b': 9, 'dlam': 10, 'A_data': 11,
}


class Params(C.Structure):
  _fields_ = [
      ('dt', f32), ('mu', f32), ('damp', f32), ('gravity', f32 * 3), ('maxiter', i32),
      ('atol', f32), ('rtol', f32), ('maxiter_cg', i32), ('tol_cg', f32), ('n_smooth', i32),
      ('omega_jacobi', f32), ('setup_interval', i32), ('use_line_search', i32), ('mode', i32),
      ('rel_tol_cg', f32), ('coarse_solver', i32), ('smoother', i32), ('max_levels', i32),
      ('max_coarse', i32), ('kinematic_pins', i32), ('coarse_sweeps', i32), ('cg_alias', i32),
      ('compliance', f32), ('precond', i32), ('cheb_degree', i32), ('cheb_lo', f32),
      ('use_graph', i32), ('persistent', i32), ('primal', i32), ('primal_tol', f32),
      ('learned_accept', f32), ('learned_stall', i32), ('cheb_scale', i32), ('body_cg', i32), ('warm_substep', i32),
  ]


class XpbdParams(C.Structure):
  """mgpbd_xpbd_params (include/mgpbd_local.h)."""
  _fields_ = [('dt', f32), ('hydro_alpha', f32), ('devia_alpha', f32), ('method', i32)]


class VbdParams(C.Structure):
  """mgpbd_vbd_params (include/mgpbd_local.h)."""
  _fields_ = [('dt', f32), ('damp', f32), ('youngs_modulus', f32), ('poissons_ratio', f32),
              ('damping', f32), ('rho', f32), ('gravity', f32 * 3), ('n_iterations', i32),
              ('method', i32)]


XPBD_METHOD = {'default': 0, 'gauss_seidel': 1, 'graph_coloring': 2}
VBD_METHOD = {'serial': 0, 'color': 1}
VBD_FIELD = {'v_v': 0, 'v_p_old': 1, 'x_tilde': 2, 'Dm_inv': 3, 'rest_vol': 4}


class Stats(C.Structure):
  _fields_ = [
      ('newton_iters', i32), ('cg_iters_total', i32), ('cg_iters_last', i32), ('n_levels', i32),
      ('residual0', f64), ('residual', f64), ('omega_last', f64), ('status', C.c_uint32),
      ('nnz', i64 * 8), ('rows', i64 * 8), ('cg_path', i32), ('cg_grid', i32),
      ('cg_iters_warm', i32), ('cg_launches', i32), ('ms_warm', f64), ('ms_dual', f64),
      ('warm_amp', f64), ('warm_declined', i32), ('learned_fallbacks', i32),
      ('learned_rejected', i32), ('learned_solves', i32), ('coarse_energy_learned', f64),
      ('coarse_energy_plain', f64),
  ]


class MGPBDError(RuntimeError):
  """A libmgpbd call returned an error code."""

  def __init__(self, code, where, detail=''):
    self.code = code
    super().__init__(f'{where}: {_strerror(code)} ({code})' + (f': {detail}' if detail else ''))


# name -> (restype, argtypes)
_SIGS = {
    'mgpbd_default_params': (None, [C.POINTER(Params)]),
    'mgpbd_strerror': (C.c_char_p, [C.c_int]),
    'mgpbd_last_error': (C.c_char_p, []),
    'mgpbd_version': (C.c_char_p, []),
    'mgpbd_launch_count': (C.c_int64, []),
    'mgpbd_create': (C.c_int, [C.POINTER(Params), C.POINTER(vp)]),
    'mgpbd_destroy': (None, [vp]),
    'mgpbd_set_stream': (C.c_int, [vp, vp]),
    'mgpbd_set_mesh': (C.c_int, [vp, vp, vp, vp, i32, i32, vp, vp]),
    'mgpbd_init': (C.c_int, [vp]),
    'mgpbd_step': (C.c_int, [vp, i32]),
    'mgpbd_make_prediction': (C.c_int, [vp]),
    'mgpbd_solve': (C.c_int, [vp, i32]),
    'mgpbd_update_vel': (C.c_int, [vp]),
    'mgpbd_get_stats': (C.c_int, [vp, C.POINTER(Stats)]),
    'mgpbd_synchronize': (C.c_int, [vp]),
    'mgpbd_get_status': (C.c_int, [vp, P_u32]),
    'mgpbd_newton_log': (C.c_int, [vp, i32, vp, P_i32]),
    'mgpbd_field': (C.c_int, [vp, i32, C.POINTER(vp), P_i64]),
    'mgpbd_level_csr': (C.c_int, [vp, i32, P_i32, P_i64, C.POINTER(vp), C.POINTER(vp),
                                  C.POINTER(vp), C.POINTER(vp)]),
    'mgpbd_level_count': (C.c_int, [vp, P_i32]),
    'mgpbd_level_agg': (C.c_int, [vp, i32, C.POINTER(vp)]),
    'mgpbd_compute_constraints': (C.c_int, [vp]),
    'mgpbd_fill_matrices': (C.c_int, [vp]),
    'mgpbd_compute_rhs': (C.c_int, [vp, P_f64]),
    'mgpbd_pcg': (C.c_int, [vp, vp, vp, P_i32]),
    'mgpbd_vcycle': (C.c_int, [vp, vp, vp]),
    'mgpbd_scatter': (C.c_int, [vp, vp]),
    'mgpbd_line_search': (C.c_int, [vp, P_f64]),
    'mgpbd_apply_dpos': (C.c_int, [vp, f64]),
    'mgpbd_apply_matrix': (C.c_int, [vp, i32, vp, vp]),
    'mgpbd_level_sweep': (C.c_int, [vp, i32, i32, vp, vp, vp, f32]),
    'mgpbd_set_hierarchy': (C.c_int, [vp, vp, i32, vp]),
    'mgpbd_set_matrix': (C.c_int, [vp, i32, C.c_int64, vp, vp, vp]),
    'mgpbd_update_matrix': (C.c_int, [vp, vp]),
    'mgpbd_set_barrier_limit': (C.c_int, [vp, C.c_double]),
    'mgpbd_set_bodies': (C.c_int, [vp, i32, vp, i32, vp]),
    'mgpbd_body_stats': (C.c_int, [vp, i32, vp, vp, vp, vp]),
    'mgpbd_zone_proximity': (C.c_int, [vp, vp, f32, f32, f32, f32]),
    'mgpbd_zone_strain': (C.c_int, [vp, vp, vp, f32, f32]),
    'mgpbd_zone_expand': (C.c_int, [vp, vp, i32]),
    'mgpbd_mask_alpha': (C.c_int, [vp, vp, vp]),
    'mgpbd_restore_alpha': (C.c_int, [vp, vp]),
    'mgpbd_host_face_adjacency': (C.c_int, [vp, i32, vp, vp, vp]),
    'mgpbd_csr_spmv': (C.c_int, [i32, vp, vp, vp, vp, vp, vp]),
    'mgpbd_csr_jacobi': (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp, f32, vp]),
    'mgpbd_csr_diag_inv': (C.c_int, [i32, vp, vp, vp, vp, vp]),
    'mgpbd_dot': (C.c_int, [i32, vp, vp, P_f64, vp]),
    'mgpbd_dot_noalloc': (C.c_int, [i32, vp, vp, P_f64, vp]),
    'mgpbd_axpy': (C.c_int, [i32, f32, vp, vp, vp]),
    'mgpbd_xpay': (C.c_int, [i32, f32, vp, vp, vp]),
    'mgpbd_scale': (C.c_int, [i32, f32, vp, vp]),
    'mgpbd_refill_coarse': (C.c_int, [vp]),
    'mgpbd_net_create': (C.c_int, [C.c_uint64, C.POINTER(vp)]),
    'mgpbd_net_destroy': (None, [vp]),
    'mgpbd_net_params': (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
    'mgpbd_net_sync_params': (C.c_int, [vp, vp]),
    'mgpbd_net_forward': (C.c_int, [vp, i32, i64, vp, vp, vp, vp, vp, vp, vp]),
    'mgpbd_net_weights': (C.c_int, [vp, i32, i64, vp, vp, vp, vp, vp, vp]),
    'mgpbd_net_apply': (C.c_int, [i32, vp, vp, vp, vp, vp]),
    'mgpbd_net_loss_grad': (C.c_int, [vp, i32, i64, vp, vp, vp, vp, vp, i32, i32, P_f64, vp]),
    'mgpbd_net_adam': (C.c_int, [vp, f32, f32, f32, f32, vp]),
    'mgpbd_net_train': (C.c_int, [vp, i32, i64, vp, vp, vp, vp, vp, i32, i32, i32, f32, vp, vp]),
    'mgpbd_set_coarse_net': (C.c_int, [vp, vp]),
    'mgpbd_set_constraint_types': (C.c_int, [vp, vp]),
    'mgpbd_row_shapes': (C.c_int, [vp, P_i32]),
    'mgpbd_autotune_rows': (C.c_int, [vp, i32, vp, vp]),
    'mgpbd_level_row_shape': (C.c_int, [vp, i32, P_i32]),
    'mgpbd_set_level_row_shape': (C.c_int, [vp, i32, i32]),
    'mgpbd_record_coarse': (C.c_int, [vp, vp, vp, i32, i32]),
    'mgpbd_record_count': (C.c_int, [vp, P_i32]),
    'mgpbd_host_pattern': (C.c_int, [vp, i32, P_i64, vp, vp]),
    'mgpbd_host_vertex_incidence': (C.c_int, [vp, i32, i32, P_i64, vp, vp]),
    'mgpbd_host_aggregate': (C.c_int, [vp, i32, i32, vp, P_i32]),
    'mgpbd_host_tet_hierarchy': (C.c_int, [vp, i32, i32, i32, P_i32, vp, vp]),
    'mgpbd_host_galerkin': (C.c_int, [i32, vp, vp, vp, vp, i32, P_i64, P_i64, vp, vp, vp, vp]),
    'mgpbd_device_galerkin': (C.c_int, [i32, vp, vp, vp, vp, i32, P_i64, P_i64, vp, vp, vp, vp,
                                        vp]),
    # include/mgpbd_local.h
    'mgpbd_color_elements': (C.c_int, [vp, i32, i32, i32, vp, vp, P_i32]),
    'mgpbd_color_vertices': (C.c_int, [vp, i32, i32, i32, vp, vp, P_i32]),
    'mgpbd_greedy_coloring': (C.c_int, [vp, vp, i32, vp, vp, P_i32]),
    'mgpbd_xpbd_create': (C.c_int, [C.POINTER(XpbdParams), C.POINTER(vp)]),
    'mgpbd_xpbd_destroy': (None, [vp]),
    'mgpbd_xpbd_set_stream': (C.c_int, [vp, vp]),
    'mgpbd_xpbd_set_mesh': (C.c_int, [vp, vp, vp, vp, vp, vp, i32, i32]),
    'mgpbd_xpbd_preupdate': (C.c_int, [vp]),
    'mgpbd_xpbd_update': (C.c_int, [vp, i32]),
    'mgpbd_xpbd_synchronize': (C.c_int, [vp]),
    'mgpbd_xpbd_lambdas': (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
    'mgpbd_xpbd_n_colors': (C.c_int, [vp, P_i32]),
    'mgpbd_vbd_create': (C.c_int, [C.POINTER(VbdParams), C.POINTER(vp)]),
    'mgpbd_vbd_destroy': (None, [vp]),
    'mgpbd_vbd_set_stream': (C.c_int, [vp, vp]),
    'mgpbd_vbd_set_mesh': (C.c_int, [vp, vp, vp, vp, vp, i32, i32]),
    'mgpbd_vbd_init': (C.c_int, [vp]),
    'mgpbd_vbd_make_prediction': (C.c_int, [vp]),
    'mgpbd_vbd_solve': (C.c_int, [vp]),
    'mgpbd_vbd_update_vel': (C.c_int, [vp]),
    'mgpbd_vbd_step': (C.c_int, [vp]),
    'mgpbd_vbd_synchronize': (C.c_int, [vp]),
    'mgpbd_vbd_omegas': (C.c_int, [vp, vp]),
    'mgpbd_vbd_field': (C.c_int, [vp, i32, C.POINTER(vp), P_i64]),
    'mgpbd_vbd_n_colors': (C.c_int, [vp, P_i32]),
    'mgpbd_vbd_lame': (C.c_int, [vp, C.POINTER(f32), C.POINTER(f32)]),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
  return _build.LIB


def lib(auto_build: bool = True):
  """Load libmgpbd.so (building it first if needed); raise if unavailable."""
  global _lib
  with _lock:
    if _lib is not None:
      return _lib
    path = _build.LIB
    if auto_build and not _build.up_to_date():
      _build.build()
    if not os.path.exists(path):
      raise OSError(f'libmgpbd.so not found at {path}; run python -m controllable_pbd_3d_gb300.build')
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
      fn = getattr(L, name)  # AttributeError if a symbol is missing
      fn.restype = res
      fn.argtypes = args
    _lib = L
    return L


def _strerror(code):
  try:
    return lib(auto_build=False).mgpbd_strerror(code).decode()
  except Exception:  # pragma: no cover - only when the library failed to load
    return 'error'


def check(code, where):
  if code != 0:
    detail = lib().mgpbd_last_error().decode()
    raise MGPBDError(code, where, detail)
  return code


def default_params() -> Params:
  p = Params()
  lib().mgpbd_default_params(C.byref(p))
  return p
