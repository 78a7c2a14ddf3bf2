"""The 1D nonstationary solver on the GPU against the reference's own runs of
nonstationary_heat_equation_solver_1d (tests/golden/d1_nonstationary_*: the
temperature after every calc_step): quadratic elements with a bell kernel,
left temperature / right flux and a sin(pi x) source from zero; linear
elements with a triangle kernel, left flux / right temperature and a sin(pi x)
initial temperature; quadratic elements with a convection at both ends
(convection_1d: heat transfer and ambient temperature).  History within 1e-10
relative L2 per step."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

SOLUTION_RTOL = 1e-10


@pytest.fixture(scope="module")
def lib():
    from nonlocal_gb300 import _lib, build
    build.build()
    _lib.load()
    if _lib.device_count() == 0:
        pytest.fail("no CUDA device visible to the nlgpu library")
    return _lib


def end(spec):
    kind = {"t": "temperature", "f": "flux", "c": "convection"}[spec[0]]
    if kind == "convection":   # c:<heat transfer>,<ambient temperature>
        h, t = spec[2:].split(",")
        return kind, (float(h), float(t))
    return kind, float(spec[2:])


@pytest.mark.parametrize("name", ["d1_nonstationary_quadratic", "d1_nonstationary_linear",
                                  "d1_nonstationary_convection"])
def test_nonstationary_1d_history(lib, name):
    from nonlocal_gb300 import thermal as T
    fx = gc.load(name)
    cfg = fx["config"]
    s = T.NonstationaryHeatEquationSolver1D(elements=int(cfg["elements"]), order=int(cfg["order"]), length=1.0,
                                            radius=float(cfg["radius"]), local_weight=float(cfg["local_weight"]),
                                            influence=cfg["influence"], conductivity=float(cfg["conductivity"]),
                                            capacity=float(cfg["capacity"]), density=float(cfg["density"]),
                                            time_step=float(cfg["dt"]))
    x = np.linspace(0.0, 1.0, s.n)
    initial = np.sin(np.pi * x) if cfg["initial"] == "sin" else None
    s.compute(left=end(cfg["left"]), right=end(cfg["right"]), initial=initial)
    if initial is not None:
        assert np.array_equal(s.temperature, initial)
    history = fx["history"]
    for k in range(history.shape[0]):
        t = s.calc_step(sin_source=cfg["source"] == "sin")
        err = np.linalg.norm(t - history[k]) / np.linalg.norm(history[k])
        assert err < SOLUTION_RTOL, (k, err)
    assert np.array_equal(s.temperature, t)


def test_nonstationary_1d_rejects_other_ends(lib):
    from nonlocal_gb300 import _lib as L
    from nonlocal_gb300 import thermal as T
    s = T.NonstationaryHeatEquationSolver1D(elements=10, order=1)
    with pytest.raises(L.NlgpuError):   # radiation ends are not built
        L.check(s.ctx._lib.nlgpu_nonstationary_1d_compute(s.ctx.handle, *s.args, L.BC_RADIATION, L.BC_FLUX, None,
                                                          None))
    with pytest.raises(L.NlgpuError):   # no compute yet
        s.calc_step(0.0, 0.0)
