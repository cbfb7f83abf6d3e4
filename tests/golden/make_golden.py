"""Generate golden vectors from the reference's own kernels (run where the reference
tree exists; the GPU host only reads the committed .npz files).

Runs, through the reference's plugin API (universe_base subclasses imported from
gravitation/kernel/), on seeded inputs:
  np1 FP32  N=1024, seed 0, 10 steps  -> per-step accelerations (float32) from np1's
            own FP32 stage 1 on its FP64 state (np1 keeps pm._r as Python floats and
            uses the base class's FP64 stage 2), plus the final state
  np1 FP64  N=1024, seed 0, 10 steps  -> accelerations of steps 0 and 9, final state
  np2 FP32  N=1024, seed 0, 10 steps  -> FP32 state after 10 steps (np2 integrates in
            FP32, np2.py:110-115), accelerations of step 0
  py1 FP64  N=128, seed 0, 5 steps    -> accelerations of step 0, final state
  galaxy    N=256 (seeded galaxy recipe, the reference's galaxy parameters, np1 FP32),
            2 steps -> accelerations of step 0
  galdev    N=300: the reference's own create_galaxy driven by the device scenario
            generator's Philox draws (pins the galaxy part of the scenario generator)
Inputs follow the uniform-cube workload: r ~ U[-1000,1000]^3, v ~ N(0,1), m ~ U[1,100]
(numpy default_rng(seed)), G, T and scaling at universe_base defaults.

Usage: python tests/golden/make_golden.py [--ref REFERENCE_TREE]
(default: $GRAVITATION_REFERENCE, else the tree oracle/build.py builds from)
"""

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from gravitation_gb300.scenarios import galaxy, uniform_cube  # noqa: E402


def run_kernel(mod, r, v, m, steps, dtype, record_a=(), **uni_kw):
    """Drive one reference kernel through universe_base, recording stage-1 output."""
    u = mod.universe(dtype=dtype, **uni_kw)
    for i in range(len(m)):
        u.add_object(name='b%d' % i, r=[float(x) for x in r[i]], v=[float(x) for x in v[i]],
                     m=float(m[i]))
    u.start()
    acc = {}
    for k in range(steps):
        # step() = stage1, stage2, stage3 (_base_.py:143-145); stage 1 output is read
        # between the stages, where the reference leaves it in pm._a
        u.step_stage1()
        if k in record_a:
            acc[k] = np.array([[float(c) for c in pm._a] for pm in u], dtype=np.float64)
        u.step_stage2()
        u.step_stage3()
    rf = np.array([[float(c) for c in pm._r] for pm in u])
    vf = np.array([[float(c) for c in pm._v] for pm in u])
    return acc, rf, vf, u


def main():
    ap = argparse.ArgumentParser()
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from oracle.build import REF_ROOT
    ap.add_argument('--ref', default=REF_ROOT)
    args = ap.parse_args()
    sys.path.insert(0, os.path.join(args.ref, 'src'))
    import importlib
    np1 = importlib.import_module('gravitation.kernel.np1')
    np2 = importlib.import_module('gravitation.kernel.np2')
    py1 = importlib.import_module('gravitation.kernel.py1')

    out = {}
    G = 6.6740831e-11
    T = 1.0e3
    r0, v0, m0 = uniform_cube(1024, seed=0)
    out['c0_r0'], out['c0_v0'], out['c0_m'] = r0, v0, m0
    out['G'], out['T'] = np.float64(G), np.float64(T)

    acc, rf, vf, u = run_kernel(np1, r0, v0, m0, 10, 'float32', record_a=range(10))
    out['np1_f32_a'] = np.stack([acc[k] for k in range(10)]).astype(np.float32)
    out['np1_f32_r10'], out['np1_f32_v10'] = rf, vf
    out['G_scaled'] = np.float64(u._G)

    acc, rf, vf, _ = run_kernel(np1, r0, v0, m0, 10, 'float64', record_a=(0, 9))
    out['np1_f64_a0'], out['np1_f64_a9'] = acc[0], acc[9]
    out['np1_f64_r10'], out['np1_f64_v10'] = rf, vf

    acc, rf, vf, _ = run_kernel(np2, r0, v0, m0, 10, 'float32', record_a=(0,))
    out['np2_f32_a0'] = acc[0].astype(np.float32)
    out['np2_f32_r10'] = rf.astype(np.float32)
    out['np2_f32_v10'] = vf.astype(np.float32)

    rs, vs, ms = uniform_cube(128, seed=0)
    out['py1_r0'], out['py1_v0'], out['py1_m'] = rs, vs, ms
    acc, rf, vf, _ = run_kernel(py1, rs, vs, ms, 5, 'float64', record_a=(0,))
    out['py1_a0'], out['py1_r5'], out['py1_v5'] = acc[0], rf, vf

    gr, gv, gmass, gpar = galaxy(256, seed=5)
    out['gal_r0'], out['gal_v0'], out['gal_m'] = gr, gv, gmass
    acc, rf, vf, ug = run_kernel(np1, gr, gv, gmass, 2, gpar['dtype'], record_a=(0,),
                                 T=gpar['T'], scale_m=gpar['scale_m'], scale_r=gpar['scale_r'])
    out['gal_np1_f32_a0'] = acc[0].astype(np.float32)
    out['gal_G_scaled'] = np.float64(ug._G)
    out['gal_T'] = np.float64(gpar['T'])
    out['gal_scale_m'] = np.float64(gpar['scale_m'])
    out['gal_scale_r'] = np.float64(gpar['scale_r'])

    out.update(reference_galaxy(args.ref, n=300, seed=5, stream=0))

    path = os.path.join(HERE, 'golden_ref.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, os.path.getsize(path), 'bytes')


def reference_galaxy(ref, n, seed, stream):
    """The reference's own create_galaxy (gravitation/lib/simulation.py:99-184, with the
    galaxy scenario's arguments, simulation.py:57-77) fed with the draws of the seeded
    device generator: for the call, random.random returns words 0, 1, 2 of Philox4x64-10
    block {body, 0} under key {seed, stream} for body 1, 2, ..., n-1 in turn (the
    uniforms the generator gives star k = body k+1).  The bodies land, scaled by
    add_object, in a reference universe_base.  simulation.py imports h5py at module
    level; the galaxy code does not use it, so a stand-in module satisfies the import."""
    import importlib
    import types
    sys.modules.setdefault('h5py', types.ModuleType('h5py'))
    sim = importlib.import_module('gravitation.lib.simulation')
    base = importlib.import_module('gravitation.kernel._base_')
    import oracle
    draws = []
    for i in range(1, n):
        w = oracle.philox4x64_10([i, 0, 0, 0], [seed, stream])
        draws += [float(int(x) >> 11) * 2.0 ** -53 for x in w[:3]]
    it = iter(draws)
    saved = sim.random.random
    sim.random.random = lambda: next(it)
    try:
        u = base.universe_base(T=2.0e12, scale_m=1.0e-30, scale_r=1.0e-10, dtype='float32')
        sim.create_galaxy(universe_obj=u, stars_len=n - 1, r=[0., 0., 0.], v=[0., 0., 0.],
                          g_alpha=0., g_beta=0., m_hole=4e40, m_star=2e30, radius=1e20)
    finally:
        sim.random.random = saved
    assert next(it, None) is None, 'create_galaxy drew a different number of uniforms'
    return {
        'galdev_r': np.array([[float(c) for c in pm._r] for pm in u._mass_list]),
        'galdev_v': np.array([[float(c) for c in pm._v] for pm in u._mass_list]),
        'galdev_m': np.array([float(pm._m) for pm in u._mass_list]),
        'galdev_G': np.float64(u._G),
        'galdev_seed': np.int64(seed), 'galdev_stream': np.int64(stream),
    }


if __name__ == '__main__':
    main()
