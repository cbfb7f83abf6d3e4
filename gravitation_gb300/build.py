"""Build libgravgb300.so in-tree with nvcc for sm_103a (GB300).

Each ``csrc/*.cu`` translation unit is compiled in parallel to ``_build/*.o`` and the
objects are linked into ``gravitation_gb300/libgravgb300.so`` against the shared CUDA
runtime.  Only sm_103a code is generated: the library refuses to run elsewhere
(grav_device_query).  Run ``python -m gravitation_gb300.build`` or call ``build()``.
"""

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
BUILD_DIR = os.path.join(HERE, '_build')
LIB_NAME = 'libgravgb300.so'
LIB_PATH = os.path.join(HERE, LIB_NAME)

ARCH_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a']
COMMON_FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC',
                '-Xcompiler', '-Wall', '--expt-relaxed-constexpr']


def _nvcc():
    cand = os.environ.get('NVCC') or shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    return cand


def _cuda_lib_dir():
    nvcc = os.path.realpath(_nvcc())
    return os.path.join(os.path.dirname(os.path.dirname(nvcc)), 'lib64')


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.h', '.cuh'))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith('.h')]
    return sorted(hs)


def source_hash():
    """Hash of every source and header (keys the autotuner cache to this build)."""
    h = hashlib.sha256()
    for p in sources() + headers():
        with open(p, 'rb') as f:
            h.update(os.path.basename(p).encode())
            h.update(f.read())
    return h.hexdigest()[:16]


def _compile(src, verbose):
    obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + '.o')
    cmd = [_nvcc()] + ARCH_FLAGS + COMMON_FLAGS + ['-I', INCLUDE, '-I', CSRC, '-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, res.stdout, res.stderr))
    return obj, res.stderr


def _up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    stamp = os.path.join(BUILD_DIR, 'stamp')
    if not os.path.exists(stamp):
        return False
    with open(stamp) as f:
        return f.read().strip() == source_hash()


def build(force=False, verbose=False, jobs=None):
    """Compile and link the library; returns its path."""
    if not force and _up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = sources()
    objs = []
    logs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or len(srcs)) as ex:
        for obj, log in ex.map(lambda s: _compile(s, verbose), srcs):
            objs.append(obj)
            logs.append(log)
    tmp = LIB_PATH + '.tmp'
    cmd = [_nvcc()] + ARCH_FLAGS + ['-shared', '-cudart', 'shared', '-o', tmp] + objs + [
        '-Xlinker', '-rpath=' + _cuda_lib_dir()]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (res.stdout, res.stderr))
    os.replace(tmp, LIB_PATH)
    with open(os.path.join(BUILD_DIR, 'stamp'), 'w') as f:
        f.write(source_hash())
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    return LIB_PATH


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
