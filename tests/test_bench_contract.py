"""bench.py's reference arm on the host cores: one JSON line with the keys the
benchmark contract names (runs the CPU restatement, no GPU), built without
the product's CUDA library, with the same `config` object as the GPU arm."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

# Runs bench.py as __main__ and, at interpreter exit, reports every shared
# object mapped into the process (the arm's whole life, since nothing is
# unmapped before exit).
_WRAPPER = r"""
import atexit, runpy, sys
def _maps():
    libs = sorted({l.split()[-1] for l in open('/proc/self/maps') if l.rstrip().endswith('.so') or '.so.' in l})
    sys.stderr.write('MAPPED_LIBS ' + ' '.join(libs) + '\n')
atexit.register(_maps)
sys.argv = [sys.argv[1]] + sys.argv[2:]
runpy.run_path(sys.argv[0], run_name='__main__')
"""


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "-c", _WRAPPER, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "1080p ms/frame" and d["unit"] == "ms/frame" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}

    # the same config object as the GPU arm prints
    sys.path.insert(0, str(ROOT))
    import bench

    assert d["config"] == bench.workload_config(1)

    # the arm ran on the oracle alone: the product library was never mapped
    mapped = [x for x in r.stderr.splitlines() if x.startswith("MAPPED_LIBS ")]
    assert len(mapped) == 1, r.stderr[-2000:]
    libs = mapped[0].split()[1:]
    assert any(x.endswith("oracle/_build/liboracle.so") for x in libs), libs
    assert not any("libmeteoros_gb300" in x for x in libs), libs


def test_gpus_n_starts_n_ranks():
    """`bench.py --gpus 2` without a launcher runs as two ranks (torchrun on
    127.0.0.1); rank 0 alone prints the line (the reference arm: host cores,
    no GPU needed)."""
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.lstrip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0][lines[0].index("{"):])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["config"]["parallelism"] == "replicas x2"
