"""The integer-pipe FP64 arithmetic of the flux kernels (fp64_int.cuh):
multiply (dmul_int), power-of-two scaling (dmul_pow2), division (ddiv_int),
square root (dsqrt_int) and the FP32<->FP64 conversions (f2d_int, d2f_int),
compiled for the host and compared bit for bit with the CPU's IEEE operations
on generated operand sets; division and square
root also with their reciprocal seeds perturbed, to show the refinement
absorbs a seed error well beyond the device's.  The GPU comparison with the
hardware operations is
tests/test_gpu_parity.py::test_integer_pipe_multiply_matches_hardware."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dmul_int_matches_ieee_multiply():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "dmul_int_host")
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "spade_gb300", "csrc"),
               os.path.join(ROOT, "tests", "cpp", "dmul_int_host.cc"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        out = subprocess.run([exe, "20000000"], capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "mismatches 0" in out.stdout
