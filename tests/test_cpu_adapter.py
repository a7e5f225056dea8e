"""The AMReX-side adapter (mesoflow_gb300/adapter/mflo_gpu_amrex.H) compiled
against the AMReX stand-in: amrex::Array4<Real> views map onto mfg_array4
element for element (padded strides, offset begins), and the flux-register
factor is the reference's scale = -+ tstep * dA * fluxfactor
(Source/mflo_evolve.cpp:662-678).  No GPU needed."""
import ctypes as C

import adapter_build


def test_array4_views_map_element_for_element():
    assert adapter_build.build(with_lib=False).adapter_view_check() == 0


def test_register_scale_is_the_references():
    lib = adapter_build.build(with_lib=True)
    dx = (C.c_double * 3)(0.1, 0.2, 0.4)
    tstep, ff = 1e-3, 1.0 / 6.0
    areas = [0.2 * 0.4, 0.1 * 0.4, 0.1 * 0.2]
    for d in range(3):
        assert lib.adapter_register_scale(-1, d, dx, tstep, ff) == -tstep * areas[d] * ff
        assert lib.adapter_register_scale(1, d, dx, tstep, ff) == tstep * areas[d] * ff
