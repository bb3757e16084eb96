"""Multi-process host logic of bench.py on CPU (gloo, world size 2).

The plain step shards by z-slabs of cells (sph_cuda_gb300.slabs, tested in
test_slabs.py), but the benchmark's headline runs one full configuration
per GPU: N GPUs run N independent replicas, and the job rate is all units
over the slowest rank's time.  The reference arm runs on rank 0
only; the other ranks exit 0 without output.
"""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, units, seconds, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rate, sec = bench.job_rate(units, seconds[rank], dist, "cpu")
        out.put((rank, rate, sec))
    finally:
        dist.destroy_process_group()


def test_job_rate_single():
    rate, sec = bench.job_rate(1000.0, 2.0)
    assert sec == 2.0 and rate == 500.0


def test_job_rate_two_ranks_takes_slowest():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    units, seconds = 4.0e6, [0.5, 0.8]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, units, seconds, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, sec in res:
        assert sec == pytest.approx(0.8)
        assert rate == pytest.approx(2 * units / 0.8)


def test_reference_arm_nonzero_rank_is_silent(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = bench.parse_args(["--impl", "reference", "--gpus", "2", "--steps", "3", "--warmup", "3"])
    buf = io.StringIO()
    with redirect_stdout(buf):
        rc = bench.run_reference(args)
    assert rc == 0 and buf.getvalue() == ""


def test_workload_presets_match_their_descriptions():
    p = bench.workload_params("bubble2m")
    assert p.n_particles == 2097152 and (p.nx, p.ny, p.nz) == (133, 133, 200)
    q = bench.workload_params("bubble524k")
    assert q.n_particles == 524288 and (q.nx, q.ny, q.nz) == (66, 66, 200)
    assert q.dx == pytest.approx(p.dx) and q.dz == pytest.approx(p.dz)


def test_reference_arm_loads_no_product_code():
    """The reference arm times the oracle port on the full configuration
    with the oracle's own parameters: it neither imports the product
    package nor maps the CUDA library."""
    import json
    import subprocess
    code = ("import sys, json; sys.path.insert(0, %r); import bench; "
            "a = bench.parse_args(['--impl', 'reference', '--workload', 'bubble524k', '--steps', '1', '--warmup', '1']); "
            "bench.run_reference(a); maps = open('/proc/self/maps').read(); "
            "print(json.dumps({'pkg': any(m.startswith('sph_cuda_gb300') for m in sys.modules), "
            "'so': 'libasph' in maps, 'oracle': 'liboracle' in maps}))" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    line, chk = lines[0], lines[-1]
    assert line["impl"] == "reference" and line["config"]["particles"] == 524288
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
    assert chk == {"pkg": False, "so": False, "oracle": True}


def test_other_workloads_and_options():
    r = bench.workload_params("reference128")
    assert (r.nx, r.ny, r.nz) == (128, 128, 128) and r.n_particles == 128 ** 3
    assert r.sort_every == 1 and r.dt_request == pytest.approx(0.25)
    big = bench.workload_params("large16m")
    assert big.n_particles == 256 ** 3 and (big.nx, big.ny, big.nz) == (250, 250, 500)
    assert big.dx / big.dz == pytest.approx(8.0)
    small = bench.workload_params("large2m")   # the large run's cells and density at 2M
    assert (small.dx, small.dz) == (big.dx, big.dz) and small.n_particles == 128 ** 3
    assert small.n_particles / (small.nx * small.ny * small.nz) == pytest.approx(
        big.n_particles / (big.nx * big.ny * big.nz))
    for name in ("bubble2m", "bubble524k", "reference128", "large16m", "large2m"):
        assert bench.workload_string(name)
        assert bench.metric_for(bench.workload_params(name)).startswith("particle-steps/s (plain step, ")
    assert bench.metric_for(bench.workload_params("bubble2m")) == bench.METRIC   # the headline metric string
    a = bench.parse_args([])
    assert a.steps == 500 and a.advance == 0 and a.workload == "bubble2m"   # the configuration's 500 steps
    assert bench.parse_args(["--advance", "500"]).advance == 500


def test_traffic_is_taken_only_from_a_capture_of_the_timed_state():
    """The roofline's DRAM traffic comes from an ncu capture of the state the
    line times: the first timed step after the warm-up, for a timed region
    short enough that the state does not drift from it."""
    r = bench.traffic_record("bubble2m", 5, 20, "density_eos")
    assert r is not None and r["steps_before"] == 5 and r["bytes"] > 48 * 2097152
    assert bench.traffic_record("bubble2m", 5, 500, "density_eos") is None     # 500 steps develop the bubbles
    assert bench.traffic_record("bubble2m", 3, 20, "density_eos") is None      # another state
    assert bench.traffic_record("bubble2m", 503, 2, "density_eos")["bytes"] > r["bytes"]
    assert bench.traffic_record("large16m", 5, 20, "density_eos") is None      # no capture of that workload
