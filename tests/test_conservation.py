"""Conservation on periodic domains, on the oracle (CPU): the flux divergence
of every scheme composition sums to round-off over a periodic box (each face
flux enters the two cells it separates with opposite signs), for the
reference-defined functors and for WENO5 / Sutherland alike.  The GPU results
equal the oracle bit for bit (tests/test_gpu_parity.py), so they conserve the
same way."""
import numpy as np
import pytest

from spade_gb300 import _abi
from oracle import oracle as O
import problems as P

CASES = {
    "ck4_visc": dict(conv=_abi.CONV_CENT_KEEP, order=4, visc=1),
    "totani_diss_visc": dict(conv=_abi.CONV_TOTANI, diss=1, visc=1),
    "fweno_ducros_visc": dict(conv=_abi.CONV_FWENO, diss=1, visc=1, sensor=_abi.SENSOR_DUCROS, alpha=0.7),
    "weno5_diss_suth": dict(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND),
    "hyb_ck2_ducros": dict(conv=_abi.CONV_HYBRID, order=2, visc=1, hybrid_sensor=_abi.SENSOR_DUCROS,
                           hybrid_param=1e-3),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_periodic_residual_sums_to_roundoff(name):
    nblk, ncell, ng = (2, 2, 1), (6, 5, 4), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, 0.0, 1.5, 0.0, 1.0))
    q = P.random_state(nblk, ncell, ng, seed=61)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    r = np.zeros_like(q)
    O.flux_div(grid, P.scheme(**CASES[name]), q, r, increment=False)
    rr = r[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    tot = np.abs(rr.sum(axis=0))
    scale = np.abs(rr).sum(axis=0)
    assert np.all(tot <= 1e-12 * np.maximum(scale, 1e-300)), tot / scale
