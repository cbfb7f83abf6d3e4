"""CPU tests of the C ABI: the library loads and exports every symbol declared in
include/*.h, the host-side planner is correct (checked by walking the persistent
kernel's work assignment in Python), and invalid arguments are rejected on the host
before anything reaches a GPU."""

import ctypes
import glob
import os
import re

import numpy as np
import pytest

from gravitation_gb300 import _lib, build as gbuild
from gravitation_gb300.engine import make_plan

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def L():
    gbuild.build()
    return _lib.load()


def header_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, 'include', '*.h')):
        src = open(h).read()
        src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
        for m in re.finditer(r'^[A-Za-z_][\w \*]*?\b(grav_\w+)\s*\(', src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_symbols_exported(L):
    names = header_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(L, name), 'symbol %s declared in include/ but not exported' % name
    # and the Python binding declares every one of them
    assert set(names) <= set(_lib.declared_symbols())


def test_abi_version(L):
    assert L.grav_abi_version() == _lib.GRAV_ABI_VERSION


def simulate_kernel(info, univ, seg, jtile):
    """Python walk of the persistent stage-1 kernel's assignment (stage1_f32.cu):
    returns (unit -> CTA) coverage and the slots each CTA writes."""
    U, G = info.n_units, info.grid
    segs = [seg[i] for i in range(info.n_seg)]
    begins = [s.unit_begin for s in segs]
    covered = np.zeros(U, dtype=np.int64)
    slots_written = {}
    for c in range(G):
        ub, ue = c * U // G, (c + 1) * U // G
        assert ub < ue
        # last segment with unit_begin <= ub
        s = max(i for i, b in enumerate(begins) if b <= ub)
        while ub < ue and s < len(segs):
            S = segs[s]
            if S.n_units == 0 or S.unit_begin + S.n_units <= ub:
                s += 1
                continue
            jt0 = ub - S.unit_begin
            jt1 = min(ue - S.unit_begin, S.n_units)
            covered[S.unit_begin + jt0:S.unit_begin + jt1] += 1
            slot = S.slot_base + (c - S.cta_first)
            assert 0 <= c - S.cta_first < S.nslots
            assert slot not in slots_written
            slots_written[slot] = (s, c)
            ub = S.unit_begin + jt1
            s += 1
    return covered, slots_written


@pytest.mark.parametrize('sizes,tile', [
    ([1], (1, 128, 128, 8)),
    ([1000], (4, 128, 256, 300)),
    ([65536], (4, 128, 256, 608)),
    ([5, 0, 300, 129, 2048], (2, 128, 128, 40)),
    ([64, 16384, 77, 1000, 3000], (4, 256, 256, 1216)),
    ([3], (8, 256, 256, 5000)),
])
def test_plan_covers_every_unit_once(L, sizes, tile):
    t = _lib.Tile(*tile)
    info, univ, seg = make_plan(sizes, 1.0, t)
    itile = t.bpt * t.threads
    assert info.itile == itile and info.pad_unit == max(itile, t.jtile)
    assert info.n_bodies == sum(sizes)
    assert info.n_pad_total == info.n_seg * itile
    assert info.grid == min(t.grid, info.n_units)
    # universes: padded, aligned, contiguous
    pad = 0
    for u, n in enumerate(sizes):
        d = univ[u]
        assert d.n == n and d.pad_off == pad and d.pad_off % info.pad_unit == 0
        assert d.n_jtiles == -(-n // t.jtile)
        pad += -(-n // info.pad_unit) * info.pad_unit
    assert pad == info.n_pad_total
    # every i-tile of real bodies has one unit per j-tile; pure padding tiles have none
    units = 0
    for s in range(info.n_seg):
        S = seg[s]
        assert S.unit_begin == units
        n = sizes[S.u]
        assert S.n_units == (univ[S.u].n_jtiles if S.il0 < n else 0)
        units += S.n_units
    assert units == info.n_units
    if info.n_units:
        covered, slots = simulate_kernel(info, univ, seg, t.jtile)
        assert np.all(covered == 1)
        assert sorted(slots) == list(range(info.n_slots))


@pytest.mark.parametrize('sizes,tile', [
    ([1], (4, 128, 128, 8)),
    ([1000], (4, 128, 128, 300)),
    ([65536], (4, 256, 256, 304)),
    ([5, 0, 3000, 129, 2048], (8, 128, 256, 40)),
    ([64, 16384, 77, 1000, 3000], (2, 256, 256, 1216)),
])
def test_pairs_plan_covers_every_pair_once(L, sizes, tile):
    """Walk grav_plan_pairs the way stage1_sym_kernel does: every row slot is written by
    exactly one CTA, and every column-slot entry of a real body exactly once."""
    t = _lib.Tile(*tile)
    info, univ, seg = make_plan(sizes, 1.0, t, 'fp32u')
    R, JT = t.bpt * t.threads, t.jtile
    TPB = R // JT
    assert info.itile == R and info.n_pad_total == info.n_seg * R
    segs = [seg[i] for i in range(info.n_seg)]
    if info.n_units == 0:
        return
    U, G = info.n_units, info.grid
    begins = [s.unit_begin for s in segs]
    written = {}
    pairs_seen = {}
    for c in range(G):
        ub, ue = c * U // G, (c + 1) * U // G
        s = max(i for i, b in enumerate(begins) if b <= ub)
        while ub < ue and s < len(segs):
            S = segs[s]
            if S.n_units == 0 or S.unit_begin + S.n_units <= ub:
                s += 1
                continue
            blkI = S.il0 // R
            t0, t1 = ub - S.unit_begin, min(ue - S.unit_begin, S.n_units)
            for tt in range(t0, t1):
                jt = blkI * TPB + tt
                blkJ = jt // TPB
                key = (S.u, blkI, jt)
                pairs_seen[key] = pairs_seen.get(key, 0) + 1
                if blkJ != blkI:
                    SJ = segs[s + blkJ - blkI]
                    assert SJ.u == S.u and SJ.il0 == blkJ * R
                    slot = SJ.slot_base + SJ.nslots - (blkJ - blkI)
                    assert SJ.slot_base <= slot < SJ.slot_base + SJ.nslots
                    off = jt * JT - blkJ * R
                    for e in range(off, off + JT):
                        written[(slot, e)] = written.get((slot, e), 0) + 1
            slot = S.slot_base + (c - S.cta_first)
            assert (slot, 'row') not in written
            written[(slot, 'row')] = 1
            ub = S.unit_begin + t1
            s += 1
    assert all(v == 1 for v in pairs_seen.values())
    assert all(v == 1 for v in written.values())
    # every slot a real body sums in stage 2 was written
    for si, S in enumerate(segs):
        n = sizes[S.u]
        nrow = S.nslots - S.il0 // R
        for k in range(S.nslots):
            slot = S.slot_base + k
            if k < nrow:
                assert (slot, 'row') in written
            else:
                for e in range(R):
                    if S.il0 + e < n:
                        assert (slot, e) in written, (si, k, e)
    # units: j-tiles from the row block onwards, real tiles only
    for u, n in enumerate(sizes):
        nb = -(-n // R)
        tiles = [k for k in pairs_seen if k[0] == u]
        assert len(tiles) == sum(univ[u].n_jtiles - I * TPB for I in range(nb))


def test_plan_rejects_bad_input(L):
    info = _lib.PlanInfo()
    n = (ctypes.c_int32 * 2)(5, -1)
    t = _lib.Tile(4, 128, 256, 10)
    assert L.grav_plan(2, n, None, ctypes.byref(t), ctypes.byref(info), None, None) == _lib.GRAV_E_ARG
    assert 'n[1]' in _lib.last_error()
    t = _lib.Tile(3, 128, 256, 10)
    n = (ctypes.c_int32 * 1)(5)
    assert L.grav_plan(1, n, None, ctypes.byref(t), ctypes.byref(info), None, None) == _lib.GRAV_E_ARG
    assert L.grav_plan(1, n, None, None, ctypes.byref(info), None, None) == _lib.GRAV_E_ARG


def test_stage_calls_reject_bad_batch_on_host(L):
    # none of these reach the GPU: validation fails first
    assert L.grav_stage1(None, None) == _lib.GRAV_E_ARG
    b = _lib.Batch()
    b.mode = 7
    assert L.grav_stage1(ctypes.byref(b), None) == _lib.GRAV_E_ARG
    assert 'mode' in _lib.last_error()
    b.mode = _lib.GRAV_MODE_FP32
    b.tile = _lib.Tile(4, 128, 256, 1)
    b.n_seg = 2
    b.n_pad_total = 1000          # != n_seg * itile
    assert L.grav_stage2(ctypes.byref(b), 1, None) == _lib.GRAV_E_ARG
    b.n_pad_total = 1024
    b.n_univ = 1
    assert L.grav_stage1(ctypes.byref(b), None) == _lib.GRAV_E_ARG   # NULL pointers
    assert L.grav_stage2(ctypes.byref(b), 0x40, None) == _lib.GRAV_E_ARG


def test_tile_table(L):
    for mode in ('fp32', 'fp32c', 'fp64'):
        m = _lib.MODES[mode]
        n = L.grav_tile_list(m, None, 0)
        assert n > 0
        arr = (_lib.Tile * n)()
        assert L.grav_tile_list(m, arr, n) == n
        for t in arr:
            assert L.grav_tile_supported(m, ctypes.byref(t)) == 1
    assert L.grav_tile_supported(0, ctypes.byref(_lib.Tile(3, 100, 7, 1))) == 0


def test_eps2_keeps_self_term_finite(L):
    for gm in (0.0, 1e-12, 6.7e-9, 1.0, 1e6, 1e12):
        e = L.grav_eps2(gm)
        assert e > 1.17549435e-38                 # a normal FP32 number
        inv = np.float32(1.0) / np.sqrt(np.float32(e))
        inv3 = inv * (inv * inv)                  # the unique-pair kernel's order
        assert np.isfinite(inv3)
        assert np.isfinite(np.float32(gm) * inv3)
        assert np.isfinite(np.float32(gm) * inv * (inv * inv))
    # far below the FP32 resolution of a unit-size separation
    assert L.grav_eps2(1.0) < 1e-20
    assert np.float32(1e-12) + np.float32(L.grav_eps2(6.7e-9)) == np.float32(1e-12)


def test_pos_and_part_bytes(L):
    assert L.grav_pos_bytes(0, 1024) == 16 * 1024
    assert L.grav_pos_bytes(1, 1024) == 32 * 1024
    assert L.grav_pos_bytes(2, 1024) == 32 * 1024
    assert L.grav_pos_bytes(9, 1024) < 0


_C_PROBE = r'''
#include <stdio.h>
#include <stddef.h>
#include "gravitation_gb300.h"

int main(void)
{
	int32_t n[2] = {1000, 37};
	double T[2] = {1e3, 2e3};
	grav_tile t = {4, 128, 128, 456};
	grav_plan_info info;
	if (grav_plan(2, n, T, &t, &info, NULL, NULL) != GRAV_OK) {
		fprintf(stderr, "%s\n", grav_last_error());
		return 1;
	}
	printf("abi %d\n", grav_abi_version());
	printf("sizes %zu %zu %zu %zu %zu %zu %zu\n", sizeof(grav_univ_desc), sizeof(grav_seg_desc),
		sizeof(grav_tile), sizeof(grav_plan_info), sizeof(grav_batch), sizeof(grav_adjoint),
		sizeof(grav_scenario));
	printf("offsets %zu %zu %zu\n", offsetof(grav_batch, univ), offsetof(grav_batch, err),
		offsetof(grav_adjoint, a_in));
	printf("plan %lld %d %d %d\n", (long long)info.n_bodies, info.n_univ, info.n_seg, info.grid);
	printf("bad %d\n", grav_plan(-1, n, T, &t, &info, NULL, NULL) == GRAV_E_ARG);
	return 0;
}
'''


def test_header_compiles_as_c_and_matches_binding(L, tmp_path):
    """The header is plain C99 (what a cgo or other FFI binding would include): a C program
    built against it with -Wall -Werror -pedantic links libgravgb300.so, calls the host-only
    entry points, and reports struct sizes and offsets equal to the ctypes mirror's."""
    import ctypes
    import shutil
    import subprocess
    if shutil.which('gcc') is None:
        pytest.skip('gcc not available')
    src = tmp_path / 'probe.c'
    src.write_text(_C_PROBE)
    exe = tmp_path / 'probe'
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(['gcc', '-std=c99', '-Wall', '-Wextra', '-Werror', '-pedantic',
                    '-I', os.path.join(ROOT, 'include'), str(src), '-o', str(exe),
                    '-L', libdir, '-lgravgb300', '-Wl,-rpath,' + libdir], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    out = dict(line.split(' ', 1) for line in res.stdout.strip().splitlines())
    assert int(out['abi']) == _lib.GRAV_ABI_VERSION
    sizes = [int(x) for x in out['sizes'].split()]
    assert sizes == [ctypes.sizeof(c) for c in (_lib.UnivDesc, _lib.SegDesc, _lib.Tile,
                                                _lib.PlanInfo, _lib.Batch, _lib.Adjoint,
                                                _lib.Scenario)]
    offs = [int(x) for x in out['offsets'].split()]
    assert offs == [_lib.Batch.univ.offset, _lib.Batch.err.offset, _lib.Adjoint.a_in.offset]
    nb, nu, nseg, grid = (int(x) for x in out['plan'].split())
    info = _lib.PlanInfo()
    t = _lib.Tile(4, 128, 128, 456)
    n_arr = (ctypes.c_int32 * 2)(1000, 37)
    T_arr = (ctypes.c_double * 2)(1e3, 2e3)
    assert L.grav_plan(2, n_arr, T_arr, ctypes.byref(t), ctypes.byref(info), None, None) == 0
    assert (nb, nu, nseg, grid) == (info.n_bodies, info.n_univ, info.n_seg, info.grid)
    assert out['bad'] == '1'


def test_fused_step_rejects_bad_calls_on_host(L):
    """grav_step_fused validates on the host (nothing reaches a GPU here)."""
    f32, f32n, f32c = _lib.GRAV_MODE_FP32, _lib.GRAV_MODE_FP32N, _lib.GRAV_MODE_FP32C
    for m in (f32, f32n, f32c):
        for threads in (256, 512, 1024):
            assert L.grav_fused_supported(m, 100, threads, 32) == 1
            assert L.grav_fused_supported(m, _lib.GRAV_FUSED_MAX_N, threads, threads) == 1
            assert L.grav_fused_supported(m, _lib.GRAV_FUSED_MAX_N + 1, threads, 32) == 0
            assert L.grav_fused_supported(m, 100, threads, threads + 1) == 0
            assert L.grav_fused_supported(m, 100, threads, 0) == 0
        assert L.grav_fused_supported(m, 100, 128, 32) == 0
    for m in (_lib.GRAV_MODE_FP64, _lib.GRAV_MODE_FP32U, _lib.GRAV_MODE_FP32UN,
              _lib.GRAV_MODE_FP32CU, 99):
        assert L.grav_fused_supported(m, 100, 256, 32) == 0
    occ = ctypes.c_int32()
    assert L.grav_fused_occupancy(f32, 100, 256, 32, None) == _lib.GRAV_E_ARG
    assert L.grav_fused_occupancy(f32, 100, 128, 32, ctypes.byref(occ)) == _lib.GRAV_E_TILE
    assert L.grav_fused_occupancy(_lib.GRAV_MODE_FP32U, 100, 256, 32,
                                  ctypes.byref(occ)) == _lib.GRAV_E_TILE
    sync = ctypes.c_void_p(16)   # never dereferenced: validation fails first
    assert L.grav_step_fused(None, 1, 256, 32, sync, None) == _lib.GRAV_E_ARG
    b = _lib.Batch()
    b.mode = f32
    b.tile = _lib.Tile(1, 128, 128, 1)
    b.n_seg, b.n_pad_total, b.n_bodies, b.n_univ = 1, 128, 100, 1
    b.univ = b.seg = b.pos = b.r = b.v = 16
    b.eps2 = 1e-25
    bb = ctypes.byref(b)
    assert L.grav_step_fused(bb, 1, 256, 32, None, None) == _lib.GRAV_E_ARG       # no sync
    assert L.grav_step_fused(bb, _lib.GRAV_S2_PREPARE, 256, 32, sync, None) == _lib.GRAV_E_ARG
    assert L.grav_step_fused(bb, _lib.GRAV_S2_WRITE_A, 256, 32, sync, None) == _lib.GRAV_E_ARG
    assert L.grav_step_fused(bb, 1, 128, 32, sync, None) == _lib.GRAV_E_TILE     # threads
    assert L.grav_step_fused(bb, 1, 256, 300, sync, None) == _lib.GRAV_E_TILE    # rows
    b.n_univ = 2
    assert L.grav_step_fused(bb, 1, 256, 32, sync, None) == _lib.GRAV_E_ARG
    assert 'one universe' in _lib.last_error()
    b.n_univ = 1
    b.mode = _lib.GRAV_MODE_FP32U
    assert L.grav_step_fused(bb, 1, 256, 32, sync, None) == _lib.GRAV_E_TILE
    b.mode = f32
    b.n_seg, b.n_pad_total, b.n_bodies = 33, 33 * 128, _lib.GRAV_FUSED_MAX_N + 1
    assert L.grav_step_fused(bb, 1, 256, 32, sync, None) == _lib.GRAV_E_SIZE


def test_eps2_is_not_a_softening_length_for_the_scenarios(L):
    """The r^2 floor grows with the heaviest G*m (it keeps G*m * r^-3 finite in FP32 at
    zero separation); for the reference's own scenarios, scaled as the universe scales
    them, sqrt(eps2) stays at least 1e6 below the closest pair's separation, so no pair
    term is softened: the galaxy (a 4e40 kg hole among 2e30 kg stars, scale_r 1e-10,
    scale_m 1e-30) and the uniform cube and Plummer pair at their SI scale."""
    from gravitation_gb300.scenarios import G_DEFAULT, galaxy, plummer_pair, uniform_cube
    r, _, m, p = galaxy(2048, seed=3)
    Gs = G_DEFAULT * p['scale_r'] ** 3 / p['scale_m']
    cases = [(r * p['scale_r'], Gs * m * p['scale_m'])]
    r, _, m = uniform_cube(2048, seed=0)
    cases.append((r, G_DEFAULT * m))
    r, _, m = plummer_pair(2048, seed=2)
    cases.append((r, G_DEFAULT * m))
    for r, gm in cases:
        eps2 = L.grav_eps2(float(gm.max()))
        d2 = ((r[:, None, :] - r[None, :, :]) ** 2).sum(-1)
        np.fill_diagonal(d2, np.inf)
        assert np.sqrt(eps2) < 1e-6 * np.sqrt(d2.min()), (eps2, d2.min())


def test_single_launch_rule_names_compiled_kernels(L):
    """The engine's size rule for the single-launch step only names compiled (mode,
    threads, rows) combinations, covers one universe of 1-512 bodies in the all-pairs
    FP32 modes, and nothing else."""
    from gravitation_gb300.engine import FUSED_MODES, default_fused
    for mode in FUSED_MODES:
        m = _lib.MODES[mode]
        for n in list(range(1, 65)) + [100, 127, 128, 129, 300, 511, 512]:
            cfg = default_fused(mode, [n])
            assert cfg is not None, (mode, n)
            threads, rows = cfg
            assert L.grav_fused_supported(m, n, threads, rows) == 1, (mode, n, cfg)
            assert -(-n // rows) <= 16        # one CTA or one thread-block cluster
        assert default_fused(mode, [513]) is None
        assert default_fused(mode, [0]) is None
        assert default_fused(mode, [100, 100]) is None
    for mode in ('fp32u', 'fp32un', 'fp32cu', 'fp64'):
        assert default_fused(mode, [100]) is None
