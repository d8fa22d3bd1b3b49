"""C-ABI checks that need no GPU: libgbns.so loads, exports every entry point
include/*.h declares, the ctypes descriptor layouts match the C structs, and
descriptor validation fails loudly before any CUDA call."""
import ctypes
import os
import re
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from spade_gb300 import _abi, _native, pde_algs, convective, viscous, viscous_laws, omni, fluid_state, state_sensor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_symbols():
    names = set()
    for f in os.listdir(INCLUDE):
        if f.endswith(".h"):
            src = open(os.path.join(INCLUDE, f)).read()
            names |= set(re.findall(r"^\s*int\s+(gbns_\w+)\s*\(", src, re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_native.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 8
    for name in syms:
        assert hasattr(lib, name), name


def test_library_version_without_gpu():
    assert _native.lib().gbns_version() == _abi.ABI_VERSION


def test_struct_layouts_match_c():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "gbns.h"
int main(void){
  printf("%zu %zu %zu %zu\n", sizeof(gbns_grid_desc), sizeof(gbns_scheme_desc), sizeof(gbns_bc_desc), sizeof(gbns_gas_desc));
  printf("%zu %zu %zu\n", offsetof(gbns_grid_desc, bounds), offsetof(gbns_scheme_desc, eps_p), offsetof(gbns_scheme_desc, gas));
  printf("%zu %zu\n", offsetof(gbns_bc_desc, t_wall), offsetof(gbns_scheme_desc, hybrid_param));
  return 0;}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I" + INCLUDE, c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [int(x) for x in out]
    want = [ctypes.sizeof(_abi.GridDesc), ctypes.sizeof(_abi.SchemeDesc), ctypes.sizeof(_abi.BcDesc), ctypes.sizeof(_abi.GasDesc),
            _abi.GridDesc.bounds.offset, _abi.SchemeDesc.eps_p.offset, _abi.SchemeDesc.gas.offset, _abi.BcDesc.t_wall.offset,
            _abi.SchemeDesc.hybrid_param.offset]
    assert got == want


def test_array_size_matches_grid_array_layout():
    g = _abi.grid_desc((2, 3, 4), (5, 6, 7), 2, (0, 1, 0, 1, 0, 1))
    n = ctypes.c_size_t(0)
    _native.check(_native.lib().gbns_array_size(g, ctypes.byref(n)))
    assert n.value == 2 * 3 * 4 * 9 * 10 * 11 * 5


@pytest.mark.parametrize("bad", ["nblk", "ng", "bounds", "coords"])
def test_invalid_grid_rejected_before_cuda(bad):
    g = _abi.grid_desc((2, 2, 2), (8, 8, 8), 2, (0, 1, 0, 1, 0, 1))
    if bad == "nblk":
        g.nblk[1] = 0
    elif bad == "ng":
        g.ng = 0
    elif bad == "bounds":
        g.bounds[3] = g.bounds[2]
    else:
        g.coords = 9
    n = ctypes.c_size_t(0)
    rc = _native.lib().gbns_array_size(g, ctypes.byref(n))
    assert rc == _abi.ERR_INVALID
    assert len(_native.last_error()) > 0


def test_flux_div_rejects_insufficient_ghosts_before_cuda():
    import problems as P
    g = _abi.grid_desc((1, 1, 1), (8, 8, 8), 2, (0, 1, 0, 1, 0, 1))
    s = P.scheme(conv=_abi.CONV_WENO5)
    rc = _native.lib().gbns_flux_div(g, s, ctypes.c_void_p(16), ctypes.c_void_p(32), 0, None)
    assert rc == _abi.ERR_INVALID
    assert "ghost" in _native.last_error()


def test_flux_div_rejects_bad_scheme_before_cuda():
    import problems as P
    g = _abi.grid_desc((1, 1, 1), (8, 8, 8), 4, (0, 1, 0, 1, 0, 1))
    s = P.scheme(conv=_abi.CONV_CENT_KEEP, order=3)
    assert _native.lib().gbns_flux_div(g, s, ctypes.c_void_p(16), ctypes.c_void_p(32), 0, None) == _abi.ERR_UNSUPPORTED
    s = P.scheme(gamma=1.0)
    assert _native.lib().gbns_flux_div(g, s, ctypes.c_void_p(16), ctypes.c_void_p(32), 0, None) == _abi.ERR_INVALID


def test_boundary_flux_validates_before_cuda():
    """gbns_boundary_flux: NULL flags, stretched coordinates and too few ghost
    layers for the ghost-row face gradients are rejected before any CUDA call."""
    import problems as P
    L = _native.lib()
    flags = (ctypes.c_int * 6)(1, 1, 1, 1, 1, 1)
    g = _abi.grid_desc((1, 1, 1), (8, 8, 8), 3, (0, 1, 0, 1, 0, 1))
    s = P.scheme(conv=_abi.CONV_WENO5, diss=1, visc=1)
    assert L.gbns_boundary_flux(g, s, ctypes.c_void_p(16), ctypes.c_void_p(32), None, None) == _abi.ERR_INVALID
    gs = _abi.grid_desc((1, 1, 1), (8, 8, 8), 3, (0, 1, -1, 1, 0, 1), coords=_abi.COORDS_TANH_Y, coord_param=(2.0, 0, 0, 0))
    assert L.gbns_boundary_flux(gs, s, ctypes.c_void_p(16), ctypes.c_void_p(32), flags, None) == _abi.ERR_UNSUPPORTED
    g1 = _abi.grid_desc((1, 1, 1), (8, 8, 8), 1, (0, 1, 0, 1, 0, 1))
    sv = P.scheme(conv=_abi.CONV_CENT_KEEP, order=2, visc=1)
    assert L.gbns_boundary_flux(g1, sv, ctypes.c_void_p(16), ctypes.c_void_p(32), flags, None) == _abi.ERR_INVALID
    assert "ghost" in _native.last_error()


def test_host_path_graph_run_and_selftest_validate_before_cuda():
    """gbns_flux_div_host (NULL or aliased arrays), gbns_ssprk3_run (negative
    step count, NULL work; zero steps is a no-op) and gbns_selftest_dmul_int
    (NULL output) fail or return before any CUDA call."""
    import problems as P
    L = _native.lib()
    g = _abi.grid_desc((1, 1, 1), (8, 8, 8), 2, (0, 1, 0, 1, 0, 1))
    s = P.scheme()
    p = ctypes.c_void_p(64)
    assert L.gbns_flux_div_host(g, s, None, p, 1, None) == _abi.ERR_INVALID
    assert L.gbns_flux_div_host(g, s, p, p, 1, None) == _abi.ERR_INVALID
    bc = _abi.BcDesc()
    assert L.gbns_ssprk3_run(g, s, bc, p, p, ctypes.c_double(1e-3), -1, None) == _abi.ERR_INVALID
    assert L.gbns_ssprk3_run(g, s, bc, p, None, ctypes.c_double(1e-3), 1, None) == _abi.ERR_INVALID
    assert L.gbns_ssprk3_run(g, s, bc, p, p, ctypes.c_double(1e-3), 0, None) == _abi.OK
    assert L.gbns_selftest_dmul_int(16, 0, None, None) == _abi.ERR_INVALID


def test_flux_div_cpu_arrays_take_the_host_path():
    """pde_algs.flux_div with grid_arrays on the CPU goes to gbns_flux_div_host
    (without a GPU: a CUDA error from the host path, never a device launch on
    host pointers); mixed CPU/GPU arguments are refused."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the host path runs (tests/test_gpu_parity.py)")
    from spade_gb300 import grid
    blocks = grid.cartesian_blocks_t((1, 1, 1), (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    g = grid.cartesian_grid_t((8, 8, 8), blocks)
    q = grid.grid_array(g, 1.0, 2, device="cpu")
    r = grid.grid_array(g, 0.0, 2, device="cpu")
    air = fluid_state.ideal_gas_t(1.4, 287.0)
    with pytest.raises(_native.SpadeError):
        pde_algs.flux_div(q, r, convective.cent_keep(2, air))


def test_fill_ghosts_rejects_unpaired_periodic():
    g = _abi.grid_desc((1, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    bc = _abi.bc_desc([_abi.BC_PERIODIC, _abi.BC_NONE, 0, 0, 0, 0])
    assert _native.lib().gbns_fill_ghosts(g, bc, ctypes.c_void_p(16), None) == _abi.ERR_INVALID


# ---------------------------------------------------------- host lowering

def air():
    return fluid_state.ideal_gas_t(1.4, 287.0)


def test_lower_compose_cent_keep_visc():
    f = omni.compose(convective.cent_keep(2, air()), viscous.visc_lr(viscous_laws.constant_viscosity_t(1e-3, 0.72), air()))
    s = pde_algs.lower(f)
    assert (s.convective, s.order, s.viscous, s.visc_law, s.dissipation) == (_abi.CONV_CENT_KEEP, 2, 1, _abi.LAW_CONSTANT, 0)
    assert s.mu == 1e-3 and s.prandtl == 0.72 and s.gas.gamma == 1.4


def test_lower_channel_composite_and_precision_trait():
    f = omni.compose(convective.weno5_t(air()),
                     convective.pressure_diss_lr(air(), state_sensor.const_sensor_t(0.5), 2.0, 3.0),
                     viscous.visc_lr(viscous_laws.sutherland_t(1e-3, 300.0, 110.4, 0.72), air()))
    s = pde_algs.lower(f, _abi.PREC_FP32_FLUX)
    assert (s.convective, s.dissipation, s.viscous, s.visc_law, s.precision) == (_abi.CONV_WENO5, 1, 1, _abi.LAW_SUTHERLAND, 1)
    assert (s.eps_p, s.eps_T, s.sensor_alpha, s.S) == (2.0, 3.0, 0.5, 110.4)


def test_lower_ducros_sensor_carries_epsilon():
    f = omni.compose(convective.fweno_t(air()),
                     convective.pressure_diss_lr(air(), state_sensor.ducros_t(1e-4), 2.0, 3.0))
    s = pde_algs.lower(f)
    assert (s.convective, s.dissipation, s.sensor) == (_abi.CONV_FWENO, 1, _abi.SENSOR_DUCROS)
    assert (s.eps_p, s.eps_T, s.sensor_alpha) == (2.0, 3.0, 1e-4)


def test_lower_rejects_noncanonical_three_term_composite():
    f = omni.compose(viscous.visc_lr(viscous_laws.constant_viscosity_t(1e-3, 0.72), air()),
                     convective.cent_keep(2, air()),
                     convective.pressure_diss_lr(air(), state_sensor.const_sensor_t(1.0), 1.0))
    with pytest.raises(_native.SpadeError):
        pde_algs.lower(f)


def test_lower_rejects_mixed_gases():
    f = omni.compose(convective.cent_keep(2, air()), viscous.visc_lr(viscous_laws.constant_viscosity_t(1e-3, 0.72),
                                                                     fluid_state.ideal_gas_t(1.3, 287.0)))
    with pytest.raises(_native.SpadeError):
        pde_algs.lower(f)


def test_cent_keep_rejects_odd_order():
    with pytest.raises(ValueError):
        convective.cent_keep(3, air())


def test_lower_hybrid_scheme():
    h = convective.hybrid_scheme_t(convective.cent_keep(4, air()), convective.fweno_t(air()),
                                   state_sensor.ducros_t(0.25), convective.diss_flux)
    s = pde_algs.lower(omni.compose(h, viscous.visc_lr(viscous_laws.constant_viscosity_t(1e-3, 0.72), air())))
    assert (s.convective, s.order, s.hybrid_flux, s.hybrid_sensor, s.hybrid_param, s.viscous) == \
        (_abi.CONV_HYBRID, 4, _abi.HYBRID_DISS_FLUX, _abi.SENSOR_DUCROS, 0.25, 1)
    with pytest.raises(ValueError):
        convective.hybrid_scheme_t(convective.cent_keep(6, air()), convective.fweno_t(air()),
                                   state_sensor.const_sensor_t(0.5), convective.full_flux)


def test_lower_sources_and_reject_callables():
    d = pde_algs.lower_source(pde_algs.body_accel_t(air(), 9.81, 0.0, -1.0))
    assert (d.kind, list(d.c), d.gas.R) == (_abi.SOURCE_BODY_ACCEL, [0.0, 0.0, 9.81, 0.0, -1.0], 287.0)
    assert pde_algs.lower_source(pde_algs.body_force_t(2.0)).kind == _abi.SOURCE_BODY_FORCE
    with pytest.raises(_native.SpadeError):
        pde_algs.lower_source(lambda q: q)
    g = _abi.grid_desc((1, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    bad = _abi.SourceDesc()
    bad.kind = 7
    assert _native.lib().gbns_source_term(g, bad, ctypes.c_void_p(16), ctypes.c_void_p(32), None) == _abi.ERR_INVALID


def test_size_limits_rejected_before_cuda():
    """The descriptor limits (64 blocks per direction; stretched-y metric
    tables of blocks_y*(ny+1) <= 1024 entries) fail with a message, not a
    fault.  The 8x8x8-block, 32^3 channel is well inside both."""
    import problems as P
    n = ctypes.c_size_t(0)
    g = _abi.grid_desc((65, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    assert _native.lib().gbns_array_size(g, ctypes.byref(n)) == _abi.ERR_INVALID
    g = _abi.grid_desc((64, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    assert _native.lib().gbns_array_size(g, ctypes.byref(n)) == _abi.OK
    g = _abi.grid_desc((1, 40, 1), (8, 32, 8), 3, (0, 1, -1, 1, 0, 1), coords=_abi.COORDS_TANH_Y, coord_param=(2.0, 0, 0, 0))
    rc = _native.lib().gbns_flux_div(g, P.scheme(conv=_abi.CONV_WENO5), ctypes.c_void_p(16), ctypes.c_void_p(32), 0, None)
    assert rc == _abi.ERR_UNSUPPORTED and "metric table" in _native.last_error()


def test_fill_array_and_physical_coordinates_on_cpu_tensors():
    """algs.fill_array evaluates a function of the physical cell centres
    (stretched y through the coordinate map) into a grid_array; CPU tensors."""
    from spade_gb300 import grid, coords, algs
    blocks = grid.cartesian_blocks_t((2, 2, 1), (0.0, 2.0, -1.0, 1.0, 0.0, 1.0))
    cs = coords.diagonal_coords(coords.identity_1D(), coords.tanh_stretch_1D(2.0), coords.identity_1D())
    g = grid.cartesian_grid_t((4, 4, 2), blocks, cs)
    q = grid.grid_array(g, 0.0, 2, device="cpu")
    algs.fill_array(q, lambda x, y, z: (x + 0 * y, y + 0 * x, z + 0 * x, 1.0, -1.0))
    d = q.data.numpy()
    ng = 2
    # x of block 1 (x-index 1), interior cell 0 = 1.0 + 0.5*0.25
    assert abs(d[1, ng, ng, ng, 0] - 1.125) < 1e-15
    # y of the first interior row of a y-min block: the stretched map of eta = -1 + 0.5*0.25
    eta = -1.0 + 0.125
    want = np.tanh(2.0 * eta) / np.tanh(2.0)
    assert abs(d[0, ng, ng, ng, 1] - want) < 1e-15
    assert np.all(d[..., 3] == 1.0) and np.all(d[..., 4] == -1.0)
    # exclude_exchanges leaves the ghosts alone
    q2 = grid.grid_array(g, 7.0, 2, device="cpu")
    algs.fill_array(q2, lambda x, y, z: (x, y, z, 0.0, 0.0), algs.exclude_exchanges)
    d2 = q2.data.numpy()
    assert np.all(d2[:, 0] == 7.0) and d2[0, ng, ng, ng, 3] == 0.0


def test_missing_library_raises_instead_of_falling_back():
    """With libgbns.so absent, the public API raises SpadeError for CPU and
    GPU grid_arrays alike: there is no CPU or PyTorch fallback.  Run in a child
    process so the loaded library of this session is untouched."""
    code = r'''
import sys
from spade_gb300 import _native, pde_algs, convective, fluid_state, grid
_native.LIB_PATH = "/nonexistent/libgbns.so"
_native._LIB = None
blocks = grid.cartesian_blocks_t((1, 1, 1), (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
g = grid.cartesian_grid_t((8, 8, 8), blocks)
q = grid.grid_array(g, 1.0, 2, device="cpu")
r = grid.grid_array(g, 0.0, 2, device="cpu")
try:
    pde_algs.flux_div(q, r, convective.cent_keep(2, fluid_state.ideal_gas_t(1.4, 287.0)))
except _native.SpadeError as e:
    assert "not built" in str(e), e
    print("raised")
    sys.exit(0)
sys.exit(1)
'''
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "raised" in r.stdout, r.stdout + r.stderr
