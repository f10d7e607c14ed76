"""The benchmark's CPU legs (the cpu_baseline sample and the reference arm)
call the oracle; run the sample on a small budget so an oracle interface
change cannot break them unnoticed."""
import bench


def test_oracle_sample_runs():
    r = bench.oracle_sample(iters=2)
    assert r["sample_nelmt"] == 6000 and r["scale"] == 32.0
    assert r["t_pcg_sample"] > 0 and r["t_stress_sample"] > 0 and r["t_plastic_iter_full"] > 0
