"""CPU tests of the tile autotuner's cache: size buckets, round trips, and robustness
against corrupt files, stale builds and entries naming tiles that are not compiled."""

import json
import types

import pytest

from gravitation_gb300 import _lib, build as gbuild
from gravitation_gb300.tune import Tuner, bucket_of

DEV = types.SimpleNamespace(name='GB300 test', sm_count=152, index=0)


@pytest.fixture(scope='module', autouse=True)
def lib():
    gbuild.build()
    return _lib.load()


def test_buckets():
    assert bucket_of([1000]) == 'single:1024'
    assert bucket_of([1024]) == 'single:1024'
    assert bucket_of([1025]) == 'single:1280'
    assert bucket_of([5000]) == 'single:5120'
    assert bucket_of([8000]) == 'single:8192'
    a, b = bucket_of([64, 128, 9000]), bucket_of([9000, 64, 128])
    assert a == b == 'batch:u4:w26:max16384'
    # the same make-up shares a key; another make-up does not
    assert bucket_of([63, 100, 9001]) == a
    assert bucket_of([64, 128, 8000]) != a
    assert bucket_of([64, 128, 9000, 9000]) != a
    # batches drawn from one distribution (other seeds) share their key
    from gravitation_gb300.scenarios import batch_universes
    keys = {bucket_of(batch_universes(256, seed)[0]) for seed in (1, 2, 3)}
    assert len(keys) <= 2, keys


def test_store_and_lookup(tmp_path):
    t = Tuner(str(tmp_path / 'c.json'), build_hash='h1')
    assert t.lookup('fp32', [4096], DEV) is None
    t.store('fp32', [4096], DEV, _lib.Tile(1, 128, 128, 512), 0.02)
    got = Tuner(str(tmp_path / 'c.json'), build_hash='h1').lookup('fp32', [4000], DEV)
    assert (got.bpt, got.threads, got.jtile, got.grid) == (1, 128, 128, 512)
    # another build of the library: the entry does not apply
    assert Tuner(str(tmp_path / 'c.json'), build_hash='h2').lookup('fp32', [4096], DEV) is None
    # another mode or size class
    assert t.lookup('fp32u', [4096], DEV) is None
    assert t.lookup('fp32', [8192], DEV) is None


def test_corrupt_and_invalid_entries(tmp_path):
    p = tmp_path / 'c.json'
    p.write_text('{not json')
    t = Tuner(str(p), build_hash='h')
    assert t.lookup('fp32', [4096], DEV) is None
    t.store('fp32', [4096], DEV, _lib.Tile(1, 128, 128, 64), 0.01)   # rewrites the file
    assert json.loads(p.read_text())['format'] == 1
    data = json.loads(p.read_text())
    key = t.key('fp32', [4096], DEV)
    for bad in ({'bpt': 3, 'threads': 128, 'jtile': 128, 'grid': 64},   # not compiled
                {'bpt': 1, 'threads': 128, 'jtile': 128, 'grid': 0},    # no grid
                {'bpt': 'x'}, 'garbage'):
        data['entries'][key] = bad
        p.write_text(json.dumps(data))
        assert Tuner(str(p), build_hash='h').lookup('fp32', [4096], DEV) is None


def test_choose_without_tuning_uses_the_cache(tmp_path):
    t = Tuner(str(tmp_path / 'c.json'), build_hash='h')
    t.store('fp32u', [65536], DEV, _lib.Tile(8, 128, 256, 456), 1.3)
    got = t.choose('fp32u', [65536], DEV, tune_if_missing=False)
    assert (got.bpt, got.threads, got.jtile, got.grid) == (8, 128, 256, 456)


def test_quarter_octave_classes():
    from gravitation_gb300.tune import fine_class
    assert [fine_class(n) for n in (0, 1, 3, 4, 5, 8, 9, 11, 13, 16, 17)] == \
        [0, 1, 3, 4, 5, 8, 10, 12, 14, 16, 20]
    assert [fine_class(n) for n in (4097, 5000, 5121, 6144, 6145, 7169, 8192)] == \
        [5120, 5120, 6144, 6144, 7168, 8192, 8192]
    for n in range(4, 70000, 37):
        c = fine_class(n)
        assert n <= c < 1.26 * n + 1, n
        assert fine_class(c) == c
