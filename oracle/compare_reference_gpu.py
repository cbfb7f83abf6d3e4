"""The reference's own GPU kernel (pc2, gravitation/kernel/pc2.py:59-91, compiled for
sm_103a by oracle/build.py) against this package's stage 1 on the same GB300 and the same
inputs (uniform cube of N bodies, seed 0): accuracy of both against the FP64 oracle on
sampled bodies, their agreement on every body, and device times.  Prints one JSON line.

Test infrastructure (a comparator), run where the pc2 cubins exist:

    python -m oracle.compare_reference_gpu [N ...]

Timings: CUDA events, L2 flushed (256 MiB write) before every timed launch, best of 5;
pc2's own step_stage1 (pc2.py:147-162) also copies the three position columns from
pageable host memory to the device and the three acceleration columns back every step,
which "pc2 stage 1 as run by the reference" times by wall clock.
"""

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle import refgpu  # noqa: E402


def main():
    import torch
    from gravitation_gb300.engine import Engine
    from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube
    from gravitation_gb300.tune import default_tuner
    sizes = [int(x) for x in sys.argv[1:]] or [1024, 4096, 16384, 65536]
    dev = torch.device('cuda', 0)
    torch.zeros(1, device=dev)
    st = torch.cuda.current_stream(dev)
    flush = torch.empty((256 << 20) // 4, dtype=torch.float32, device=dev)

    def timed(fn, reps=5):
        best = None
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            t = e0.elapsed_time(e1)
            best = t if best is None else min(best, t)
        return best

    out = []
    for n in sizes:
        if not refgpu.available(n):
            out.append({'n': n, 'skipped': 'no pc2 cubin for this N (built where the '
                        'reference tree exists)'})
            continue
        r, v, m = uniform_cube(n, seed=0)
        f32 = dict(dtype=torch.float32, device=dev)
        cols = [torch.tensor(r[:, k], **f32) for k in range(3)]
        acc = [torch.zeros(n, **f32) for _ in range(3)]
        mm = torch.tensor(m, **f32)
        k = refgpu.Pc2Kernel(n)
        h = st.cuda_stream

        def pc2():
            k.launch(*(t.data_ptr() for t in cols), *(t.data_ptr() for t in acc),
                     mm.data_ptr(), h)
        pc2()
        torch.cuda.synchronize()
        a_pc2 = torch.stack(acc, 1).double().cpu().numpy()
        mode = 'fp32u' if n >= 8192 else 'fp32'
        eng = Engine([n], 1e3, mode=mode, tuner=default_tuner())
        eng.set_state(r, v, G_DEFAULT * m)
        a_ours = eng.forces().cpu().numpy()
        rows = np.random.default_rng(11).choice(n, min(n, 128), replace=False)
        r32 = r.astype(np.float32).astype(np.float64)
        ref = oracle.accel_fp64(r32, (G_DEFAULT * m.astype(np.float32).astype(np.float64)),
                                1.0, rows=rows, coincident=True)
        t_pc2 = timed(pc2)
        t_s1 = timed(eng.stage1)
        t_step = timed(lambda: eng.step(1))
        # pc2's stage 1 as the reference runs it: pageable F-order host columns up, the
        # kernel, the accelerations down, synchronously (pc2.py:147-162)
        host_r = np.asfortranarray(r.astype(np.float32))
        host_a = np.zeros((n, 3), dtype=np.float32, order='F')
        walls = []
        for _ in range(5):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for c in range(3):
                cols[c].copy_(torch.from_numpy(host_r[:, c]))
            pc2()
            for c in range(3):
                host_a[:, c] = acc[c].cpu().numpy()
            walls.append(time.perf_counter() - t0)
        out.append({
            'n': n, 'mode': mode,
            'pc2_kernel_ms': t_pc2, 'pc2_interactions_per_s': n * n / (t_pc2 * 1e-3),
            'pc2_stage1_with_copies_ms': 1e3 * min(walls),
            'ours_stage1_ms': t_s1, 'ours_stage1_interactions_per_s': n * n / (t_s1 * 1e-3),
            'ours_step_ms': t_step, 'ours_step_interactions_per_s': n * n / (t_step * 1e-3),
            'speedup_stage1_vs_pc2_kernel': t_pc2 / t_s1,
            'max_rel_err_pc2_vs_fp64_oracle': float(oracle.rel_err_per_body(a_pc2[rows], ref).max()),
            'max_rel_err_ours_vs_fp64_oracle': float(oracle.rel_err_per_body(a_ours[rows], ref).max()),
            'max_rel_diff_ours_vs_pc2_all_bodies': float(oracle.rel_err_per_body(a_ours, a_pc2).max()),
        })
        k.close()
        del eng
    print(json.dumps({'comparison': 'reference pc2 kernel vs gravitation_gb300 stage 1 on one GB300',
                      'results': out}))
    return 0


if __name__ == '__main__':
    sys.exit(main())
