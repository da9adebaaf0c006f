"""Build the engine's shared library in-tree with nvcc (sm_103a only).

    python -m probability_gb300.build

Compiles every ``csrc/*.cu`` translation unit in parallel into
``probability_gb300/lib/libgb300mcmc.so``.  The library has a plain C ABI
(``include/gb300_mcmc.h``) and no Python or torch dependency.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
LIBDIR = os.path.join(HERE, 'lib')
LIBNAME = 'libgb300mcmc.so'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc():
  cand = os.environ.get('NVCC') or shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
  if not os.path.exists(cand):
    raise RuntimeError('nvcc not found; set NVCC or put CUDA 13 on PATH')
  return cand


def cuda_libdir(cc):
  """lib64 of the CUDA toolkit that owns `cc` (runtime path of cuBLAS)."""
  return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(cc))), 'lib64')


def sources():
  return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _flags(extra=()):
  return (ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
                  '-Xcompiler', '-fvisibility=hidden', '-I', INCLUDE, '-I', CSRC,
                  '--expt-relaxed-constexpr'] + list(extra))


def build(verbose=False, ptxas_info=False):
  os.makedirs(LIBDIR, exist_ok=True)
  objdir = os.path.join(LIBDIR, 'obj')
  os.makedirs(objdir, exist_ok=True)
  cc = nvcc()
  extra = ['-Xptxas', '-v'] if ptxas_info else []

  def compile_one(src):
    obj = os.path.join(objdir, os.path.basename(src)[:-3] + '.o')
    cmd = [cc, '-c', src, '-o', obj] + _flags(extra)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, ' '.join(cmd), r.stderr))
    if verbose or ptxas_info:
      sys.stderr.write(r.stderr)
    return obj

  srcs = sources()
  with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
    objs = list(ex.map(compile_one, srcs))
  out = os.path.join(LIBDIR, LIBNAME)
  tmp = out + '.tmp'
  cmd = [cc, '-shared', '-o', tmp] + objs + ARCH + ['-lcudart', '-lcublas',
                                                     '-Xlinker', '-rpath=' + cuda_libdir(cc)]
  r = subprocess.run(cmd, capture_output=True, text=True)
  if r.returncode != 0:
    raise RuntimeError('link failed:\n%s\n%s' % (' '.join(cmd), r.stderr))
  os.replace(tmp, out)
  return out


if __name__ == '__main__':
  print(build(verbose='-v' in sys.argv, ptxas_info='--ptxas' in sys.argv))
