"""Host-side set-up of the benchmark workloads (no GPU)."""
import numpy as np

from hydrothermal3d_gb300 import hrl


def test_ensemble_workload_generator():
    mem = hrl.ensemble(n_members=6, seed=4)
    assert len(mem) == 6
    sizes = set()
    for T, P, ktv, kfv, p in mem:
        nx, ny, nz = (s - 2 for s in T.shape)
        sizes.add((nx, ny, nz))
        assert all(31 <= v <= 95 for v in (nx, ny, nz))
        assert 100.0 <= p.Ra <= 5000.0
        assert kfv.shape == (nx + 1, ny + 1, nz + 1) and kfv.min() > 0 and np.isfinite(kfv).all()
        assert abs(np.log10(kfv).std() - 0.25) < 0.05
        assert p.thermal.nitout == mem[0][4].thermal.nitout
    assert len(sizes) == 6
    # seeded: the same members again
    again = hrl.ensemble(n_members=6, seed=4)
    for a, b in zip(mem, again):
        np.testing.assert_array_equal(a[3], b[3])
        assert a[4].Ra == b[4].Ra


def test_dt_max_caps_the_adapted_dt(orc):
    """dt_max bounds the adapted dt (0 keeps the reference's unbounded rule)."""
    n = 8
    T, P, ktv, kfv = hrl.initial_fields(n, n, n, seed=3)
    dts = []
    for cap in (0.0, 1e-5):
        p = hrl.params(n, n, n, Ra=100.0, nitout=100, dt_max=cap)
        V = [np.zeros((n + 1, n, n), order="F"), np.zeros((n, n + 1, n), order="F"), np.zeros((n, n, n + 1), order="F")]
        Tc, Pc = T.copy(order="F"), P.copy(order="F")
        s, _, _ = orc.step_hrl(Tc, Pc, ktv, kfv, *V, p)
        assert s == 0
        dts.append(p.dt)
    assert dts[0] > 1e-5 and dts[1] == 1e-5


def test_curl_velocity_is_discretely_divergence_free():
    import torch
    from hydrothermal3d_gb300 import sweep
    for n in ((12, 9, 7), (16, 16, 16)):
        V = sweep.curl_velocity(*n, seed=6, device="cpu")
        assert V[0].shape == (n[0] + 1, n[1], n[2]) and V[0].stride() == (1, n[0] + 1, (n[0] + 1) * n[1])
        assert float(sweep.divergence(*V).abs().max()) < 1e-12 * max(n)
        assert abs(max(float(v.abs().max()) for v in V) - 1.0) < 1e-14
        # no flow through the walls
        assert float(V[0][0].abs().max()) < 1e-14 and float(V[0][-1].abs().max()) < 1e-13
        assert float(V[1][:, 0].abs().max()) < 1e-14 and float(V[2][:, :, -1].abs().max()) < 1e-13
    a = sweep.curl_velocity(8, 8, 8, seed=6, device="cpu")[1]
    b = sweep.curl_velocity(8, 8, 8, seed=6, device="cpu")[1]
    assert torch.equal(a, b)


def test_fault_slab_case():
    import torch
    T, P, ktv, kfv, p = hrl.fault_slab_case(n=21, device="cpu")
    assert T.shape == (23, 23, 23) and kfv.shape == (22, 22, 22) and p.dt_max == 1e-3
    ratio = float(kfv[9:13].mean() / torch.cat([kfv[:8], kfv[14:]]).mean())
    assert 5.0 < ratio < 20.0  # the x10 slab over a log-normal background
    assert abs(float(torch.log10(kfv[:8]).std()) - 0.25) < 0.08
    inner = T[1:-1, 1:-1, 1:-1]
    assert float(inner.max()) <= 1.0 + 1e-3 and float(inner.min()) >= -1e-3


def test_bench_command_line():
    """bench.py parses its default and documented options without a GPU."""
    import importlib.util
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_cli", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    argv = sys.argv
    try:
        sys.argv = ["bench.py"]
        a = bench.parse()
        assert (a.gpus, a.impl, a.n) == (1, "ours", 255) and a.warmup >= 3
        sys.argv = ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3", "--mixed-refresh", "1024",
                    "--nu-steps", "0", "--post-n", "0", "--fault-steps", "20"]
        a = bench.parse()
        assert a.impl == "reference" and a.mixed_refresh == 1024 and a.fault_steps == 20
        c = bench.workload_config(a)
        assert c["cells"] == 255 ** 3 and c["mixed_refresh"] == 1024
    finally:
        sys.argv = argv
