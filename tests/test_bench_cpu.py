"""The benchmark's CPU legs (the cpu_baseline sample and the reference arm)
call the oracle; run the sample on a small budget so an oracle interface
change cannot break them unnoticed."""
import bench


def test_oracle_sample_runs():
    r = bench.oracle_sample(iters=2)
    assert r["sample_nelmt"] == 6000 and r["scale"] == 32.0
    assert r["t_pcg_sample"] > 0 and r["t_stress_sample"] > 0 and r["t_plastic_iter_full"] > 0


def test_admission_report_counts_requests_held_by_the_budget():
    """A request that waits while a worker is idle was held by the HBM budget;
    one that starts the moment a worker frees was held by the worker count."""
    one = [dict(t_arrival=0.0, t_start=0.0, t_done=10.0, footprint=1e9),
           dict(t_arrival=1.0, t_start=10.0, t_done=20.0, footprint=1e9)]
    r = bench.admission_report(one, 1, 2e9)
    assert r["held_by_budget_with_idle_worker"] == 0 and r["peak_running_footprint_gb"] == 1.0
    two = [dict(t_arrival=0.0, t_start=0.0, t_done=10.0, footprint=1.5e9),
           dict(t_arrival=1.0, t_start=10.0, t_done=20.0, footprint=1.5e9)]
    r = bench.admission_report(two, 2, 2e9)
    assert r["held_by_budget_with_idle_worker"] == 1 and r["budget_gb"] == 2.0


def test_pcg_count_comes_from_the_oracle_record():
    n, src = bench.pcg_count_ref()
    assert n == 860.0 and "oracle" in src
