"""bench.py's reference arm on the CPU: it runs the oracle port on the host
cores, prints the contract's JSON line with the same `config` as the
engine's arm would, and loads no library of the engine."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_line_and_libraries():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--side", "8", "--steps", "2",
                        "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "spring-updates/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    libs = line["native_libraries"]
    assert libs is not None and not any(x.startswith("titan_gb300/") for x in libs), libs
    sys.path.insert(0, str(ROOT))
    import bench
    assert line["config"] == bench.workload_config(8, 512, line["config"]["springs"], 1)
