"""C ABI checks that need no GPU: the library loads, exports every entry
point declared in include/*.h, and its host-side layout reproduces the
reference's MSR pattern bit for bit."""
import os
import re

import numpy as np
import pytest

from goma_gb300 import _lib
from goma_gb300.newton import msr_pattern_host
from tests import golden_cases as gc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from goma_gb300 import build
        build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) > 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("name", gc.names())
def test_host_msr_pattern_matches_reference(lib, name):
    g, case = gc.load(name)
    ija = msr_pattern_host(gc.problem_from_case(case))
    assert np.array_equal(ija, g["ija"])


def test_host_layout_rejects_bad_connectivity(lib):
    from goma_gb300 import problem as pb
    prob = pb.lid_cavity_2d(2)
    prob.mesh.conn = prob.mesh.conn.copy()
    prob.mesh.conn[1, 3] = prob.mesh.num_nodes + 5
    with pytest.raises(_lib.GbError, match="outside"):
        msr_pattern_host(prob)


def test_newton_options_fill_the_abi_struct(lib):
    """gb_newton_opts_default needs no device; named options land in the C
    struct (fp32_inner as linear_precision) and an unknown name is an error."""
    import types

    from goma_gb300.newton import GomaNewton
    host = types.SimpleNamespace(_L=lib)
    o = GomaNewton.newton_opts(host, krylov_dim=45, forcing=1, fp32_inner=True, linear_tol=1e-9)
    assert (o.krylov_dim, o.forcing, o.linear_precision, o.linear_tol) == (45, 1, 1, 1e-9)
    d = GomaNewton.newton_opts(host)
    assert d.linear_precision == 0 and d.max_newton > 0
    with pytest.raises(TypeError, match="krylov"):
        GomaNewton.newton_opts(host, krylov=30)


def test_abi_struct_mirrors_match_the_library(lib):
    """The ctypes mirrors of the ABI structs have the library's sizes, and
    the Newton options' defaults land in the right fields."""
    import ctypes

    from goma_gb300 import problem as pb
    assert lib.gb_abi_struct_size(0) == ctypes.sizeof(_lib.NewtonOpts)
    assert lib.gb_abi_struct_size(1) == ctypes.sizeof(_lib.NewtonStats)
    assert lib.gb_abi_struct_size(2) == ctypes.sizeof(pb.CProblemDesc)
    assert lib.gb_abi_struct_size(3) == ctypes.sizeof(pb.CMaterial)
    assert lib.gb_abi_struct_size(99) == 0
    o = _lib.NewtonOpts()
    lib.gb_newton_opts_default(ctypes.byref(o))
    assert (o.max_newton, o.krylov_dim, o.max_refinements, o.forcing) == (20, 30, 20, 0)
    assert (o.inner_tol, o.forcing_max, o.factorization_reuse) == (1e-3, 1e-2, 0)
