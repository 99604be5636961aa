"""The served loop on the GPU: every job's result is the same alone and in
the mix (exactly: a job's kernels read and write only its own mesh, and the
per-mesh arithmetic does not depend on what else runs at the same time), the
device-driven stop rule agrees with the host-driven plain path, and
admission respects the HBM budget."""

import numpy as np
import pytest

from gpumesh_gb300 import serve

pytestmark = pytest.mark.gpu


def small_stream():
    return serve.poisson_stream(rate=400.0, seconds=0.06, seed=4, lo=300, hi=20000)


def test_same_result_alone_and_in_the_mix():
    stream = small_stream()
    assert len(stream) >= 12
    server = serve.Server(keep_results=True)
    mix = server.run(stream, realtime=False)
    assert mix.peak_active > 3  # jobs really overlapped on the device
    picks = [j for j in stream if j.job_id % 4 == 0][:6]
    assert {j.smoother for j in picks} >= {"nelder_mead", "gradient_descent"}
    for spec in picks:
        alone = serve.Server(keep_results=True).run([spec], realtime=False)
        a, m = alone.results[spec.job_id], mix.results[spec.job_id]
        assert a["passes"] == m["passes"]
        assert np.array_equal(a["pos"], m["pos"])
        assert a["min"] == m["min"] and a["mean"] == m["mean"]
    server.close()


def test_device_stop_rule_matches_the_host_driven_plain_path():
    stream = small_stream()[:10]
    server = serve.Server(keep_results=True)
    served = server.run(stream, realtime=False)
    plain = serve.run_plain(server, stream, realtime=False)
    for spec in stream:
        s, p = served.results[spec.job_id], plain.results[spec.job_id]
        assert s["passes"] == p["passes"], spec
        assert np.array_equal(s["pos"], p["pos"])
        assert s["min"] == p["min"] and s["mean"] == p["mean"]
    assert served.relocations == plain.relocations
    server.close()


def test_admission_respects_the_budget():
    stream = small_stream()[:8]
    s = serve.Server(hbm_budget_bytes=1)  # room for one job at a time
    stats = s.run(stream, realtime=False)
    assert stats.peak_active == 1
    assert stats.jobs == 8 and len(stats.latencies_s) == 8
    s.close()


def test_stop_rule_and_pass_cap():
    stream = small_stream()[:6]
    s = serve.Server(max_passes=3, keep_results=True)
    stats = s.run(stream, realtime=False)
    for r in stats.results.values():
        assert 1 <= r["passes"] <= 3
    s.close()


def test_slots_are_reused_across_jobs():
    stream = small_stream()
    s = serve.Server()
    s.run(stream, realtime=False)
    created = s.slots_created
    s.run(stream, realtime=False)  # the same jobs again: every slot already exists
    assert s.slots_created == created
    s.close()
