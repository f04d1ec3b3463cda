"""CPU: bench.py's reference arm and its launcher, end to end.

- `--gpus 2` without a launcher's environment starts two ranks itself
  (torch.distributed.run on 127.0.0.1); rank 0 alone runs the CPU arm and
  prints one line, with n_gpus 2;
- the reference arm's `config` has the same keys and values as the GPU
  arm's for the same workload;
- the reference arm maps nothing of the GPU library (its tables come from
  the oracle's tabulation).
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _json_lines(out: str):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_reference_arm_two_ranks_self_launched():
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2",
                        "--impl", "reference", "--workload", "mass_p3", "--cells", "256",
                        "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["config"]["parallelism"] == "replicas2"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["flags"]
    assert line["value"] > 0


def test_reference_arm_config_matches_gpu_arm_and_loads_no_gpu_library():
    code = r"""
import io, json, sys, contextlib
sys.path.insert(0, ROOT)
import bench
from femtc_gb300 import workloads as W
import oracle

class A: pass
a = A()
a.workload, a.cells, a.steps, a.warmup = "stiffness_p4", 64, 1, 3
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.run_reference(a, 0, 1)
line = json.loads(buf.getvalue())
w = W.make("stiffness_p4", ncells=64, tabulate=oracle.tabulate)
same = line["config"] == bench.workload_config(w, 1, 8)
maps = open("/proc/self/maps").read()
print(json.dumps({"same": same, "gpu_lib": "libfemtc_gpu" in maps,
                  "oracle_fast": "liboracle_fast" in maps}))
""".replace("ROOT", repr(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["same"]
    assert not res["gpu_lib"]
    assert res["oracle_fast"]
