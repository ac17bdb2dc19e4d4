"""The N > 1 bench path on CPU: two `gloo` ranks, each timing its own
requests.  The job's time is the maximum over ranks and its throughput the
pixels of all ranks over that time; each rank serves its own pose set."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "ngp-encode-server_gb300"))
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        local_ms = 100.0 * (rank + 1)  # rank 1 is the slower one
        job = bench.job_time_ms(local_ms, w)
        poses = bench.rank_poses(r)
        q.put((r, w, local, job, bench.job_mrays(w, 1920 * 1080, 10, job), [list(p) for p in poses[:2]]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_and_throughput():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, job0, mr0, poses0), (r1, w1, l1, job1, mr1, poses1) = out
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert job0 == job1 == pytest.approx(200.0)        # max over ranks
    assert mr0 == mr1 == pytest.approx(2 * 1920 * 1080 * 10 / 0.2 / 1e6)  # all ranks' pixels over that time
    assert poses0 != poses1                             # each rank serves its own requests


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.job_time_ms(12.5, 1) == 12.5
    assert bench.job_mrays(1, 100, 4, 1000.0) == pytest.approx(400 / 1.0 / 1e6)


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` (the CPU restatement of the path on the
    host cores; no GPU) prints exactly one JSON line with the keys the
    contract names, its e2e equal to its value and no host-device bytes."""
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("reference", "port") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun only rank 0 runs the reference arm; the others exit 0
    without output."""
    import subprocess
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=300, cwd=REPO, env=env)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_maps_no_product_library():
    """The reference arm times the CPU restatement only: the process maps the
    oracle's library and never the CUDA library, and its `config` is the
    one the GPU arm prints."""
    import json
    import subprocess
    code = ("import sys, json, argparse; sys.argv=['bench.py']; sys.path.insert(0, %r); import bench; "
            "a = argparse.Namespace(gpus=1, steps=1, warmup=0); bench.run_reference(a); "
            "maps = open('/proc/self/maps').read(); "
            "print(json.dumps({'nes': 'libnes_gb300' in maps, 'oracle': 'liboracle' in maps, "
            "'config': bench.bench_config()}))" % REPO)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    line, probe = lines[0], lines[-1]
    assert probe["oracle"] and not probe["nes"]
    assert line["config"] == probe["config"]


def test_oracle_focal_matches_library(nes_lib):
    import oracle
    for w in (1, 33, 400, 800, 1280, 1920, 4096):
        for fov in (45.5, 60.0, 90.0, 100.0, 120.0):
            assert oracle.focal_from_fov(w, fov) == nes_lib.focal_from_fov(w, fov)


def test_roofline_terms_gather_on_l1_pipe(monkeypatch):
    """The gather term is the L1 data pipe's wavefront rate over its peak
    (one wavefront per SM per cycle at the sampled clock); `bound` names
    the term with the larger floor, and the line's frac is that term's."""
    sys.path.insert(0, REPO)
    import bench
    monkeypatch.setitem(bench.L1_WF_PER_SAMPLE, ("fp16", 13), 20.0)
    n, ms = 1e8, 10.0
    head = {"march_ms": ms, "raygen_ms": 0.01, "samples_per_step": n, "ms_per_step": ms,
            "clocks": {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0}, "rays_per_step": 1000}
    out = bench.roofline_terms(head, "fp16", 1700.0, "measured", 7000.0, 100, 13)
    wf_rate = 20.0 * n / (ms / 1e3)
    frac = wf_rate / (100 * 2000e6)
    assert out["gather"]["frac"] == pytest.approx(frac, rel=1e-3)
    assert out["gather"]["floor_ms"] == pytest.approx(ms * frac, rel=1e-3)
    gbs = n * 512 / (ms / 1e3) / 1e9
    assert out["gather"]["peak"] == pytest.approx(gbs / frac, rel=1e-3)
    tflops = n * bench.FLOP_PER_SAMPLE / (ms / 1e3) / 1e12
    assert out["tensor"]["frac"] == pytest.approx(tflops / 1700.0, rel=1e-3)
    assert out["bound"] == "gather" and out["frac"] == out["gather"]["frac"]
    # Without a wavefront figure for the configuration only the tensor term is placed.
    out = bench.roofline_terms(head, "fp16", 1700.0, "measured", 7000.0, 100, 10)
    assert out["bound"] == "tensor" and "gather" not in out
