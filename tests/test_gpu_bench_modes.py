"""bench.py's side modes on small inputs: `--flux-variants` (one plain
flux_div per tile variant, the launch sequence the ncu summaries capture)
prints one JSON line with a time and a rate for every variant the library
reports, for each workload and both precisions; `--batch-only` prints the
batched form's block."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload", ["taylor_green", "channel", "channel_fweno"])
@pytest.mark.parametrize("precision", ["fp64", "fp32_flux"])
def test_flux_variants_mode(workload, precision):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--flux-variants", workload, "--precision", precision,
           "--nblk", "2", "1", "1", "--ncell", "16", "16", "16", "--steps", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["flux_variants"] == workload and line["cells"] == 2 * 16 ** 3
    times = line["ms_per_variant"]
    assert len(times) >= 2 and all(t > 0 for t in times.values())
    assert str(line["best"]) in times


def test_batch_only_mode():
    """`--batch-only` prints the batched form's block: both precisions, the
    autotuned variant per class and a positive rate."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--batch-only", "--batch-instances", "4", "--batch-steps", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    block = json.loads(r.stdout.strip().splitlines()[-1])["batch_form"]
    assert block["instances"] == 4 and block["steps"] == 2
    for prec in ("fp64", "fp32_flux"):
        assert block[prec]["cell_steps_per_s"] > 0
        assert all(t["variant"] >= 0 for t in block[prec]["autotuned"].values())
