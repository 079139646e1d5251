"""The bench on the CPU: its N > 1 path, which runs independent replicas (the
field step has no collective: each GPU runs a replica of the problem),
where two gloo ranks take the barrier and the maximum of their times and the
reference arm runs on rank 0 alone; the reference arm's JSON line; and the
clock summary of the timed region."""
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(r, port, q):
    os.environ.update({"RANK": str(r), "LOCAL_RANK": str(r), "WORLD_SIZE": "2", "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch
    import bench
    bench.init_dist(torch)
    bench.barrier()
    # each replica's time; the job's time is the slowest replica's
    got = bench.max_over_ranks(1.5 + r)
    q.put((r, bench.world(), bench.rank(), got))
    bench._dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    assert out == [(0, 2, 0, 2.5), (1, 2, 1, 2.5)]


def test_reference_arm_runs_on_rank_zero_alone():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_line_keeps_the_contract():
    # the reference arm (the oracle port on the host's cores) prints one JSON
    # line with the arm's metric, a cpu_baseline describing the run and an e2e
    # of its own value with no host-device copies
    import json
    env = dict(os.environ)
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["value"] > 0 and d["unit"] == "node-steps/s" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["same_config"] is True
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]


def test_clock_summary_reads_the_timed_region():
    # the bench's nvidia-smi summary: the median SM clock and the largest max
    # clock of the samples inside the timed region, the throttle reasons any
    # of them had active, malformed lines left out; with no sample inside, the
    # first one after the region, counted as trailing
    sys.path.insert(0, ROOT)
    import bench
    c = bench.Clocks(0)
    na, on = "Not Active", "Active"
    c.samples = [(0.5, ["1400", "2070", "300", na, na, na, na]),
                 (1.1, ["2070", "2070", "900", na, na, na, on]),
                 (1.2, ["2050", "2070", "950", na, na, na, na]),
                 (1.3, ["[N/A]", "2070", "950", na, na, na, na]),
                 (1.35, ["2070", "2070"]),
                 (1.4, ["2070", "2070", "990", na, na, na, na]),
                 (2.5, ["2070", "2070", "100", on, na, na, na])]
    c.t0, c.t1 = 1.0, 2.0
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 4 and s["trailing_samples"] == 0
    c.t0, c.t1 = 2.0, 2.2
    s = c.summary()
    assert s["samples"] == 0 and s["trailing_samples"] == 1 and s["reasons"] == ["hw_slowdown"]
