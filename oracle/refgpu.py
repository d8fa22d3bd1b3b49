"""The reference's own GPU flux_div, run on this GPU.  TEST INFRASTRUCTURE ONLY.

The reference's CUDA path (pde-algs/flux-div/flux_div.h:16-56 with the
basic, bfoct and longf algorithms; dispatch/execute.h) cannot be compiled on
a machine without the reference's sources.  It is therefore run in two
halves:

* where the sources are (``record_all``): oracle/refgpu/ref_gpu_harness.cu is
  compiled against them twice, as a host program linked with a recording
  stand-in for the CUDA runtime (oracle/refgpu/record_cudart.cc) and as a
  cubin.  Running the host program once per case below writes a launch
  script: the reference's own allocations, geometry uploads and kernel
  launches with their argument bytes, for one flux_div per algorithm.
* on the GPU (``Replay``): oracle/refgpu/replay.cc loads the cubin, relocates
  the recorded device addresses to real allocations (the prims and rhs
  arrays are the caller's tensors, in the same AoS5 grid_array layout) and
  launches the reference's kernels unchanged.

Only tests/ and bench.py's reference legs use this module.
"""
import ctypes
import math
import os
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
CUBIN = os.path.join(REF_DIR, "ref_gpu.cubin")
RECORDER = os.path.join(REF_DIR, "ref_gpu_record")
REPLAY_LIB = os.path.join(REF_DIR, "libref_gpu_replay.so")

TWO_PI = 2.0 * math.pi


def _cases():
    """The cases the reference's GPU flux_div is recorded for, each the
    nearest scheme the reference can run to a benchmark workload, at the
    benchmark's size (8x8x8 blocks of 32^3 = 16.8M cells):

    * tgv_ck2_visc: the Taylor-Green configuration's scheme,
      compose(cent_keep<2>, visc_lr(constant)), 2 ghost layers;
    * channel_fweno_diss_visc: the channel with the schemes the reference
      has (fweno_t, pressure_diss_lr(const_sensor), visc_lr(constant)) on a
      uniform grid, 2 ghost layers (bfoct needs exactly 2)."""
    import sys
    sys.path.insert(0, os.path.dirname(_HERE))
    from spade_gb300 import fluid_state, pde_algs, workloads
    air = fluid_state.ideal_gas_t(1.4, 287.0)
    u0, mu_tgv = workloads.tgv_params()
    c_w, U_b, mu_ch = workloads.channel_params()
    s_ch = pde_algs.lower(workloads.channel_flux(air, mu_ch, c_w, weno="fweno", law="constant"))
    return {
        "tgv_ck2_visc": dict(scheme="ck2_visc", nblk=(8, 8, 8), ncell=(32, 32, 32), ng=2,
                             bounds=(0.0, TWO_PI, 0.0, TWO_PI, 0.0, TWO_PI), gamma=1.4, R=287.0,
                             mu=mu_tgv, prandtl=0.72, eps_p=0.0, eps_T=0.0, sensor=0.0,
                             algs=("basic", "bfoct", "longf")),
        "channel_fweno_diss_visc": dict(scheme="fweno_diss_visc", nblk=(8, 8, 8), ncell=(32, 32, 32), ng=2,
                                        bounds=(0.0, 4 * math.pi, -1.0, 1.0, 0.0, 4 * math.pi / 3),
                                        gamma=1.4, R=287.0, mu=s_ch.mu, prandtl=s_ch.prandtl,
                                        eps_p=s_ch.eps_p, eps_T=s_ch.eps_T, sensor=s_ch.sensor_alpha,
                                        algs=("basic", "bfoct", "longf")),
    }


CASE_NAMES = ("tgv_ck2_visc", "channel_fweno_diss_visc")


def script_path(case):
    return os.path.join(REF_DIR, "refgpu_%s.rec" % case)


def available():
    """True when the cubin and every recorded launch script are present."""
    return os.path.exists(CUBIN) and all(os.path.exists(script_path(c)) for c in CASE_NAMES)


def record_all(ref_src):
    """Builds the recorder and the cubin from the reference's sources and
    writes one launch script per case (no GPU needed)."""
    subprocess.run(["make", "-s", "-C", _HERE, "refgpu", "REF_SRC=" + ref_src], check=True)
    for name, c in _cases().items():
        args = [RECORDER, c["scheme"]] + [str(x) for x in c["nblk"]] + [str(x) for x in c["ncell"]] + [str(c["ng"])]
        args += ["%.17g" % x for x in c["bounds"]]
        args += ["%.17g" % c[k] for k in ("gamma", "R", "mu", "prandtl", "eps_p", "eps_T", "sensor")]
        args += [",".join(c["algs"])]
        out = script_path(name)
        env = dict(os.environ, REFREC_OUT=out + ".tmp")
        subprocess.run(args, check=True, env=env)
        os.replace(out + ".tmp", out)


def _lib():
    if not os.path.exists(REPLAY_LIB):
        subprocess.run(["make", "-s", "-C", _HERE, "refgpu-replay"], check=True)
    L = ctypes.CDLL(REPLAY_LIB)
    vp, cp = ctypes.c_void_p, ctypes.c_char_p
    L.refgpu_open.argtypes = [cp, cp, ctypes.c_char_p, ctypes.c_size_t]
    L.refgpu_open.restype = vp
    L.refgpu_error.argtypes = [vp]
    L.refgpu_error.restype = cp
    L.refgpu_bind.argtypes = [vp, cp, ctypes.c_ulonglong, ctypes.c_ulonglong]
    L.refgpu_prepare.argtypes = [vp, vp]
    L.refgpu_nphases.argtypes = [vp]
    L.refgpu_phase_name.argtypes = [vp, ctypes.c_int]
    L.refgpu_phase_name.restype = cp
    L.refgpu_phase_launches.argtypes = [vp, ctypes.c_int]
    L.refgpu_run.argtypes = [vp, ctypes.c_int, vp]
    L.refgpu_close.argtypes = [vp]
    return L


class Replay:
    """One recorded case bound to the caller's prims and rhs device arrays
    (torch float64 tensors in the AoS5 layout with ghosts)."""

    def __init__(self, case, prims, rhs, stream):
        self.L = _lib()
        err = ctypes.create_string_buffer(512)
        self.h = self.L.refgpu_open(script_path(case).encode(), CUBIN.encode(), err, 512)
        if not self.h:
            raise RuntimeError("reference GPU replay: " + err.value.decode())
        self._check(self.L.refgpu_bind(self.h, b"prims", prims.data_ptr(), prims.numel() * 8))
        self._check(self.L.refgpu_bind(self.h, b"rhs", rhs.data_ptr(), rhs.numel() * 8))
        self._check(self.L.refgpu_prepare(self.h, stream))
        self.phases = {self.L.refgpu_phase_name(self.h, i).decode(): i for i in range(self.L.refgpu_nphases(self.h))}
        self.launches = {k: self.L.refgpu_phase_launches(self.h, i) for k, i in self.phases.items()}

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference GPU replay: " + self.L.refgpu_error(self.h).decode())

    def run(self, alg, stream):
        """Enqueues the reference's flux_div of algorithm `alg` (increment
        mode: rhs += divergence) on `stream`."""
        self._check(self.L.refgpu_run(self.h, self.phases[alg], stream))

    def close(self):
        if self.h:
            self.L.refgpu_close(self.h)
            self.h = None

    def __del__(self):
        self.close()
