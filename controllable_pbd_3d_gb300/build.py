"""Build `libmgpbd.so` in-tree for sm_103a (GB300).

    python -m controllable_pbd_3d_gb300.build [--force] [--debug-bounds]

Each translation unit under `csrc/` is compiled in parallel (nvcc for `.cu`,
g++ with OpenMP for the host structure builders) into `_build/`, then linked
into `controllable_pbd_3d_gb300/libmgpbd.so`.  A rebuild happens only when a
source or header is newer than the library.
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libmgpbd.so')
INCLUDE = os.path.join(os.path.dirname(PKG), 'include')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _nvcc():
  for cand in (shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
    if cand and os.path.exists(cand):
      return cand
  raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libmgpbd.so')


def _sources():
  return sorted(glob.glob(os.path.join(CSRC, '*.cu')) + glob.glob(os.path.join(CSRC, '*.cpp')))


def _deps():
  return _sources() + glob.glob(os.path.join(CSRC, '*.h')) + glob.glob(
      os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(INCLUDE, '*.h')) + [__file__]


def up_to_date() -> bool:
  if not os.path.exists(LIB):
    return False
  t = os.path.getmtime(LIB)
  return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src, extra):
  nvcc = _nvcc()
  obj = os.path.join(BUILD, os.path.basename(src) + '.o')
  if src.endswith('.cu'):
    cmd = [nvcc, '-std=c++17', *ARCH, '-O3', '-lineinfo', '-Xcompiler', '-fPIC,-fopenmp',
           '-I' + INCLUDE, *extra, '-c', src, '-o', obj]
  else:
    cmd = ['g++', '-std=c++17', '-O2', '-fPIC', '-fopenmp', '-I' + INCLUDE, *extra, '-c', src,
           '-o', obj]
  r = subprocess.run(cmd, capture_output=True, text=True)
  if r.returncode != 0:
    raise RuntimeError(f'compile failed: {" ".join(cmd)}\n{r.stdout}\n{r.stderr}')
  return obj


def build(force: bool = False, extra=(), verbose: bool = False) -> str:
  """Compile every CUDA/C++ source and link libmgpbd.so; returns its path."""
  if not force and up_to_date():
    return LIB
  os.makedirs(BUILD, exist_ok=True)
  srcs = _sources()
  with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
    objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
  tmp = LIB + '.tmp'
  cmd = [_nvcc(), '-shared', *ARCH, '-o', tmp, *objs, '-Xcompiler', '-fopenmp', '-lgomp']
  r = subprocess.run(cmd, capture_output=True, text=True)
  if r.returncode != 0:
    raise RuntimeError(f'link failed: {" ".join(cmd)}\n{r.stdout}\n{r.stderr}')
  os.replace(tmp, LIB)
  if verbose:
    print(f'built {LIB}')
  return LIB


def main(argv=None):
  ap = argparse.ArgumentParser()
  ap.add_argument('--force', action='store_true')
  a = ap.parse_args(argv)
  build(force=a.force, verbose=True)


if __name__ == '__main__':
  sys.exit(main())
