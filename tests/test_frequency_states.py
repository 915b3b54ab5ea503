"""CPU: the frequency-state prefetchers that feed the sweeps (solver_gb300/frequency.py):
states built by spawned worker processes or a worker thread equal the direct
construction, and several threads walking the sequence concurrently (as the port lanes
do) each get every state once it is built, with release() dropping kept states."""
import threading

import numpy as np
import pytest

from solver_gb300 import configs, frequency as fq, mesher


@pytest.fixture(scope="module")
def crossbar():
    out, freqs, _settings, z0, _grid = mesher.parse_request(configs.crossbar_20x20x4())
    esc, inc, _cc, diag, _exp, ports, le, _li, Zs = out
    static = (esc, inc, diag, Zs, le, ports, z0)
    ws = 2 * np.pi * np.array([1e8, 1e9, 3e9]) * esc["freq"]
    return static, ws


def _walk(pf, seq, out, lane):
    for pos, k in enumerate(seq):
        out.append((lane, k, pf.get(k, pos)))


@pytest.mark.parametrize("kind", ["pool", "thread"])
def test_concurrent_walkers_get_every_state(crossbar, kind):
    static, ws = crossbar
    seq = [0, 1, 2, 1]
    if kind == "pool":
        pf = fq.FrequencyPool(static, lambda k: ws[k], seq, workers=2, lookahead=2, keep=True)
    else:
        pf = fq.StatePrefetcher(lambda k: fq.FrequencyState(ws[k], *static), seq, keep=True)
    try:
        got = []
        th = [threading.Thread(target=_walk, args=(pf, seq, got, i)) for i in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert len(got) == 2 * len(seq)
        for _lane, k, st in got:
            ref = fq.FrequencyState(ws[k], *static)
            np.testing.assert_array_equal(st.DZ, ref.DZ)
            assert abs(st.w - ws[k]) == 0
        pf.release(1)
        assert pf.get(1).DZ.shape == got[0][2].DZ.shape  # rebuilt on demand
    finally:
        pf.close()
