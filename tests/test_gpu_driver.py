"""Time-loop driver (hydrothermal3d_gb300/driver.py): per-step JSON lines with
the Nusselt number and solver statistics, restart files every nout steps, and
a restart that continues bit for bit like the uninterrupted run."""
import json

import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import abi, api, driver, hrl

pytestmark = pytest.mark.gpu
N = 16


def fields():
    T, P, ktv, kfv = hrl.initial_fields(N, N, N, seed=1)
    V = [ht.zeros(N + 1, N, N), ht.zeros(N, N + 1, N), ht.zeros(N, N, N + 1)]
    return [ht.from_numpy(a) for a in (T, P, ktv, kfv)] + [V]


def test_log_breakpoints_and_restart(ctx, tmp_path):
    T, P, ktv, kfv, V = fields()
    p = hrl.params(N, N, N, dt_max=2e-3)
    log = tmp_path / "run.jsonl"
    recs = driver.run_hrl(ctx, T, P, ktv, kfv, V, p, 4, abi.MIXED, log=str(log), nout=2, out_dir=str(tmp_path))
    lines = [json.loads(x) for x in log.read_text().splitlines()]
    assert [r["it"] for r in lines] == [1, 2, 3, 4] and lines == json.loads(json.dumps(recs))
    for r in lines:
        assert r["thermal"]["status"] == 0 and r["darcy"]["status"] == 0 and r["thermal"]["iters"] > 0
        assert abs(r["Nu"] - 1.0) < 0.05  # near-conductive start of the HRL run
        assert 0.0 <= r["T_min"] <= r["T_max"] <= 1.0 + 1e-3
    assert (tmp_path / "Breakpoint00002.h5").exists() and (tmp_path / "Breakpoint00004.h5").exists()
    # restart from step 2: steps 3 and 4 again, identical to the first run
    T2, P2, _, _, V2 = fields()
    q = hrl.params(N, N, N, dt_max=2e-3)
    recs2 = driver.run_hrl(ctx, T2, P2, ktv, kfv, V2, q, 2, abi.MIXED, out_dir=str(tmp_path), restart_from=2)
    assert [r["it"] for r in recs2] == [3, 4]
    assert np.array_equal(ht.to_numpy(T2), ht.to_numpy(T)) and np.array_equal(ht.to_numpy(P2), ht.to_numpy(P))
    assert recs2[-1]["time"] == recs[-1]["time"] and recs2[-1]["Nu"] == recs[-1]["Nu"]


def test_nusselt_of_the_conductive_state(ctx):
    """Pure conduction (Ra = 0 in effect: T = 1 - y, no perturbation): Nu = 1."""
    T, P, ktv, kfv = hrl.initial_fields(N, N, N, seed=1, amp=0.0)
    p = hrl.params(N, N, N)
    probe = driver.NusseltProbe(ctx, N, N, N)
    assert abs(probe(ht.from_numpy(T), ht.from_numpy(ktv), p) - 1.0) <= 1e-12
