"""Build recipe for the CPU oracle (test infrastructure only).

Builds, with gcc, next to this file:
  liboracle.so  -- oracle.c: FP64 all-pairs oracle, FP64 stage 2, energy, adjoint check;
                   scenario.c: the seeded scenario generator restated
  libport.so    -- ref_port.c: portable restatement of the reference's fastest CPU
                   stage 1 (the timed CPU baseline)
and, only where the reference tree is present (this is never the case on the GPU
host), compiles the reference's own sources where they lie, into ``oracle/_ref/``:
  _ref/lib1.so  -- gravitation/kernel/_lib1_/lib.c (the c1a kernel), with the
                   reference's own flags (setup.py:82-99)
  _ref/cy4/     -- gravitation/kernel/cy4/core.pyx through Cython (setup.py:73-78)
  _ref/pc2_n<N>.cubin -- the CUDA kernel of gravitation/kernel/pc2.py (its SM string,
                   pc2.py:59-91), rendered as pc2's start_kernel renders it for FP32 and
                   N bodies (pc2.py:125-131) and compiled with nvcc for sm_103a: the
                   reference's own GPU kernel, as a comparator on the GB300 (a cubin is
                   device code only, so it serves the GPU host as built here)
The reference's _lib4_/lib.c (c4a/c4b) is not built: it includes x86 SSE headers
(lib.c:39) and GCC 13 rejects its OpenMP data-sharing clause (lib.c:179-182).

Usage: ``python oracle/build.py`` or ``oracle.build.build_all()``.
"""

import os
import platform
import shutil
import subprocess
import sys
import sysconfig
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference's source tree: $GRAVITATION_REFERENCE, else where this build recipe
# finds it in the development container (absent on the GPU host, where only the builds
# made from it travel)
REF_ROOT = os.environ.get('GRAVITATION_REFERENCE') or '/root/reference'
REF_KERNEL = os.path.join(REF_ROOT, 'src', 'gravitation', 'kernel')
# the reference's Python package staged into the repository's git-ignored baseline/_ref
# (sources included), so that it travels with the repository to the GPU host, where the
# reference tree itself does not exist; its C and Cython kernels are compiled there
BASELINE_REF = os.path.join(os.path.dirname(HERE), 'baseline', '_ref')
STAGED_KERNEL = os.path.join(BASELINE_REF, 'gravitation', 'kernel')


def _run(cmd):
    subprocess.run(cmd, check=True)


def _newer(target, *sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False):
    out = os.path.join(HERE, 'liboracle.so')
    srcs = [os.path.join(HERE, 'oracle.c'), os.path.join(HERE, 'scenario.c')]
    if force or not _newer(out, *srcs):
        _run(['gcc', '-O2', '-fPIC', '-shared', '-fopenmp', '-ffp-contract=off',
              '-std=gnu11', '-Wall'] + srcs + ['-o', out, '-lm'])
    return out


def build_port(force=False):
    out = os.path.join(HERE, 'libport.so')
    src = os.path.join(HERE, 'ref_port.c')
    if force or not _newer(out, src):
        # the reference's own optimisation flags (setup.py:103-118) minus the
        # x86-only -march=native / -mfpmath=sse
        _run(['gcc', '-O3', '-ffast-math', '-fPIC', '-shared', '-fopenmp',
              '-std=gnu11', '-Wall', src, '-o', out, '-lm'])
    return out


def reference_flags():
    """The reference's C optimisation flags (setup.py:103-118) on this host."""
    flags = ['-O3', '-ffast-math']
    if platform.machine() in ('x86_64', 'AMD64'):
        flags += ['-march=native', '-mtune=native', '-mfpmath=sse']
    return flags


def build_port_reference_flags(force=False):
    """ref_port.c compiled with exactly the reference's flags on this host (x86:
    -march=native etc.), into oracle/_ref/, for a like-for-like comparison with the
    reference's own C kernel; the timed baseline uses the portable build_port()."""
    refdir = os.path.join(HERE, '_ref')
    os.makedirs(refdir, exist_ok=True)
    out = os.path.join(refdir, 'libport_refflags.so')
    src = os.path.join(HERE, 'ref_port.c')
    if force or not _newer(out, src):
        _run(['gcc'] + reference_flags() + ['-fPIC', '-shared', '-fopenmp', '-std=gnu11',
                                            src, '-o', out, '-lm'])
    return out


def reference_present():
    return os.path.isfile(os.path.join(REF_KERNEL, '_base_.py'))


def stage_reference(force=False):
    """Where the reference tree is present: copy its Python package (src/gravitation,
    sources included, no build products) to baseline/_ref/gravitation and render cy4's
    Cython source to C beside it (cy4/core.c: the GPU host has no Cython).  pip cannot
    install the reference offline on GCC 13: its c4a extension (_lib4_/lib.c, x86 SSE)
    fails to compile (default(none) without PHY_G_SSE, lib.c:179-182), which stops the
    whole build.  Returns the staged package directory, or None."""
    if not reference_present():
        return None
    src = os.path.join(REF_ROOT, 'src', 'gravitation')
    dst = os.path.join(BASELINE_REF, 'gravitation')
    stamp = os.path.join(BASELINE_REF, '.staged')
    if force or not os.path.isfile(stamp):
        shutil.rmtree(dst, ignore_errors=True)
        shutil.copytree(src, dst, ignore=shutil.ignore_patterns('*.so', '__pycache__', '*.pyc'))
        with open(stamp, 'w') as f:
            f.write(src + '\n')
    # click, the reference front end's one pure-Python dependency that the GPU host lacks,
    # from the local wheelhouse (the other absent imports have stand-ins, oracle/standins)
    wheels = os.environ.get('GRAVITATION_WHEELHOUSE') or '/opt/wheelhouse'
    if not os.path.isdir(os.path.join(BASELINE_REF, 'click')) and os.path.isdir(wheels):
        try:
            _run([sys.executable, '-m', 'pip', 'install', '--quiet', '--no-index', '--no-deps',
                  '--find-links', wheels, '--target', BASELINE_REF, 'click'])
        except (subprocess.CalledProcessError, OSError):
            pass
    pyx = os.path.join(dst, 'kernel', 'cy4', 'core.pyx')
    c_file = os.path.join(dst, 'kernel', 'cy4', 'core.c')
    if os.path.isfile(pyx) and (force or not _newer(c_file, pyx)):
        try:
            _run([sys.executable, '-m', 'cython', '-3', pyx, '-o', c_file])
        except (subprocess.CalledProcessError, OSError):
            pass
    return dst


def staged_reference():
    """True when baseline/_ref holds the staged reference package."""
    return os.path.isfile(os.path.join(STAGED_KERNEL, '_base_.py'))


def build_reference(force=False):
    """Compile the reference's c1a C kernel and cy4 Cython kernel, on this host, from the
    staged reference package (stage_reference; here, or on the GPU host after the push):
    in place, where the reference's own wrappers load them (_lib1_/lib.so, cy4/core*.so),
    and as copies in oracle/_ref/ (lib1.so, cy4/core*.so).  The reference's compiler
    flags are used (setup.py:87-118) minus the x86-only ones on other hosts.

    Returns a dict name -> path (or an error string) for what was attempted.
    """
    result = {}
    stage_reference()
    if not staged_reference():
        return result
    refdir = os.path.join(HERE, '_ref')
    os.makedirs(refdir, exist_ok=True)
    lib1_src = os.path.join(STAGED_KERNEL, '_lib1_', 'lib.c')
    lib1_inplace = os.path.join(STAGED_KERNEL, '_lib1_', 'lib.so')
    lib1_out = os.path.join(refdir, 'lib1.so')
    try:
        if force or not _newer(lib1_inplace, lib1_src):
            flags = ['-std=gnu11', '-fPIC', '-Wall'] + reference_flags()
            _run(['gcc'] + flags + ['-shared', lib1_src, '-o', lib1_inplace, '-lm'])
        shutil.copyfile(lib1_inplace, lib1_out)
        result['lib1'] = lib1_out
    except (subprocess.CalledProcessError, OSError) as e:
        result['lib1'] = 'unbuildable: %s' % e
    cy4_dir_src = os.path.join(STAGED_KERNEL, 'cy4')
    cy4_c = os.path.join(cy4_dir_src, 'core.c')
    suffix = sysconfig.get_config_var('EXT_SUFFIX')
    cy4_inplace = os.path.join(cy4_dir_src, 'core' + suffix)
    cy4_dir = os.path.join(refdir, 'cy4')
    cy4_out = os.path.join(cy4_dir, 'core' + suffix)
    try:
        if not os.path.isfile(cy4_c):
            raise OSError('cy4/core.c not rendered (no Cython where the package was staged)')
        if force or not _newer(cy4_inplace, cy4_c):
            inc = sysconfig.get_paths()['include']
            _run(['gcc', '-O3', '-fPIC', '-shared', '-fopenmp', '-I', inc,
                  cy4_c, '-o', cy4_inplace, '-lm'])
        os.makedirs(cy4_dir, exist_ok=True)
        shutil.copyfile(cy4_inplace, cy4_out)
        result['cy4'] = cy4_out
    except (subprocess.CalledProcessError, OSError) as e:
        result['cy4'] = 'unbuildable: %s' % e
    return result


PC2_SIZES = (1024, 4096, 16384, 65536)


def _pc2_template():
    """The SM source template of pc2.py (a module-level string), read without importing
    the module (it needs PyCUDA)."""
    import ast
    src = os.path.join(REF_KERNEL, 'pc2.py')
    tree = ast.parse(open(src).read())
    for node in tree.body:
        if isinstance(node, ast.Assign) and any(
                isinstance(t, ast.Name) and t.id == 'SM' for t in node.targets):
            return ast.literal_eval(node.value)
    raise ValueError('no SM template in %s' % src)


def build_reference_gpu(sizes=PC2_SIZES, G=6.6740831e-11, force=False):
    """Compile pc2's kernel for each N in `sizes` (FP32, int32 indices, rsqrtf, the
    universe's G: the values pc2.py:125-131 formats in) into oracle/_ref/pc2_n<N>.cubin.
    PyCUDA's SourceModule compiles its source inside extern "C", so the rendered source
    is wrapped the same way and the kernel keeps its plain name, update_all."""
    result = {}
    if not reference_present():
        return result
    refdir = os.path.join(HERE, '_ref')
    os.makedirs(refdir, exist_ok=True)
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    src_py = os.path.join(REF_KERNEL, 'pc2.py')
    try:
        tmpl = _pc2_template()
    except (OSError, ValueError, SyntaxError) as e:
        return {'pc2': 'unbuildable: %s' % e}
    for n in sizes:
        out = os.path.join(refdir, 'pc2_n%d.cubin' % n)
        try:
            if force or not _newer(out, src_py):
                code = tmpl.format(dtype='float', itype='int32', rsqrt='rsqrtf', G=G,
                                   MASS_LEN=int(n))
                with tempfile.TemporaryDirectory() as tmp:
                    cu = os.path.join(tmp, 'pc2_kernel.cu')
                    with open(cu, 'w') as f:
                        f.write('extern "C" {\n' + code + '\n}\n')
                    _run([nvcc, '-cubin', '-O3', '-gencode', 'arch=compute_103a,code=sm_103a',
                          cu, '-o', out])
            result['pc2_n%d' % n] = out
        except (subprocess.CalledProcessError, OSError) as e:
            result['pc2_n%d' % n] = 'unbuildable: %s' % e
    return result


def build_all(force=False):
    out = {'oracle': build_oracle(force), 'port': build_port(force)}
    out.update(build_reference(force))
    out.update(build_reference_gpu(force=force))
    return out


def clean_reference():
    shutil.rmtree(os.path.join(HERE, '_ref'), ignore_errors=True)


if __name__ == '__main__':
    for k, v in build_all(force='--force' in sys.argv).items():
        print(k, v)
