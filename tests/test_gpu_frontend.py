"""The reference's own front end drives gb1 on the GB300: its `benchmark` command runs one
`worker` subprocess per size over its galaxy scenario (the reference's unseeded
generator, its universe parameters), and its `analyze` command parses and validates the
log (oracle/frontend.py; the reference package staged in baseline/_ref, stand-ins for the
imports this host lacks)."""

import pytest

pytestmark = pytest.mark.gpu


def test_reference_benchmark_and_analyze_drive_gb1(gpu, tmp_path):
    from oracle import frontend
    ok, why = frontend.available()
    if not ok:
        pytest.skip(why)
    data, log, _ = frontend.run(6, 8, str(tmp_path), min_iterations=3, min_total_runtime=1)
    rows = frontend.summary(data)
    # the reference's size range 2^6 .. 2^8 with its interpolated sizes (cli/benchmark.py
    # _range), each a galaxy of that many bodies
    stars = [64, 96, 128, 192, 256]
    assert [r['n'] for r in rows] == stars, rows
    for r in rows:
        assert r['kernel'] == 'gb1'
        assert r['steps'] >= 3 and 0 < r['best_ns'] <= r['mean_ns']
    text = open(log).read()
    assert text.count('{"log": "EXIT", "msg": "OK"}') == len(stars)
