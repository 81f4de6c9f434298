"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point declared in include/sphgrid.h, and its host functions
(mappingParameters, output sizes, error reporting) agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(sphg_[a-z_0-9]+)\s*\(",
                                    src, re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared_symbols()
    for must in ("sphg_map", "sphg_context_create", "sphg_context_destroy",
                 "sphg_mapping_parameters", "sphg_last_error", "sphg_output_len"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    lib = C.CDLL(os.path.join(ROOT, "sphtogrid.jl_gb300", "libsphgrid.so"))
    missing = [n for n in _declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.sphg_abi_version() == 1


PARAM_CASES = [
    dict(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256),
    dict(center=[3.0, 3.0, 3.0], x_size=6.0, y_size=6.0, z_size=6.0, Npixels=500),
    dict(center=[0.1, -0.3, 7.0], x_size=0.7, y_size=1.3, z_size=2.0, pixelSideLength=0.013),
    dict(x_lim=[-64, 64], y_lim=[-64, 64], z_lim=[-64, 64], Npixels=200, boxsize=100.0),
    dict(center=[0.0, 0.0, 0.0], x_lim=[-1.0, 1.0], y_lim=[-1.0, 1.0], z_lim=[-1.0, 1.0],
         pixelSideLength=0.2),
]


@pytest.mark.parametrize("kw", PARAM_CASES)
def test_mapping_parameters_match_oracle(pkg, oracle, kw):
    p = pkg.mappingParameters(**kw)
    o = oracle.mapping_parameters(**kw).as_dict()
    assert p.x_lim == o["x_lim"] and p.y_lim == o["y_lim"] and p.z_lim == o["z_lim"]
    assert p.center == o["center"] and p.halfsize == o["halfsize"]
    assert p.len2pix == o["len2pix"] and p.pixelSideLength == o["pixelSideLength"]
    assert p.Npixels == o["Npixels"] and p.boxsize == o["boxsize"] and p.periodic == o["periodic"]


def test_mapping_parameters_errors(pkg):
    # runtests.jl:38-58
    with pytest.raises(pkg.SPHtoGridError, match="Giving a center position requires extent") as e:
        pkg.mappingParameters()
    assert e.value.status == 1
    with pytest.raises(pkg.SPHtoGridError, match="Please specify pixelSideLength or number of pixels!"):
        pkg.mappingParameters(center=[0.0, 0.0, 0.0], x_lim=[-1.0, 1.0], y_lim=[-1.0, 1.0],
                              z_lim=[-1.0, 1.0])


def test_output_len(pkg):
    from sphtogrid_gb300 import _lib
    par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=16)
    o = _lib.SphgOptions()
    o.dimensions = 2
    assert _lib.lib().sphg_output_len(C.byref(par._c), C.byref(o), 3) == 16 * 16 * 3
    o.return_both_maps = 1
    assert _lib.lib().sphg_output_len(C.byref(par._c), C.byref(o), 3) == 16 * 16 * 4
    o.dimensions = 3
    assert _lib.lib().sphg_output_len(C.byref(par._c), C.byref(o), 1) == 16 ** 3
    o.dimensions = 4
    assert _lib.lib().sphg_output_len(C.byref(par._c), C.byref(o), 1) == -1


def test_bad_dimensions_centre_and_return_none(pkg):
    # cic_interpolation.jl:59,148-272: centring happens, then `nothing`
    par = pkg.mappingParameters(center=[1.0, 1.0, 1.0], x_size=2.0, y_size=2.0, z_size=2.0,
                                Npixels=4)
    pos = np.asfortranarray(np.ones((3, 2)))
    one = np.ones(2)
    out = pkg.sphMapping(pos, one, one, one, one, param=par, kernel=pkg.Cubic(),
                         dimensions=4, show_progress=False)
    assert out is None
    assert np.array_equal(pos, np.zeros((3, 2)))


def test_faraday_branch_rejected(pkg):
    par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=4)
    pos = np.asfortranarray(np.full((3, 1), 0.5))
    one = np.ones(1)
    with pytest.raises(NotImplementedError):
        pkg.sphMapping(pos, one, one, one, one, one, one, param=par, kernel=pkg.Cubic(),
                       show_progress=False)


def test_no_device_is_reported(pkg):
    """Without a GPU, creating a context fails with SPHG_ERR_NO_DEVICE (there is
    no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.SPHtoGridError) as e:
        pkg.Context(0)
    assert e.value.status == 10


def test_differentiable_precision_is_validated(pkg):
    """An unknown forward or adjoint precision is rejected before any device
    work."""
    import torch
    par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=4)
    t = torch.ones(1, dtype=torch.float64)
    pos = torch.full((3, 1), 0.5, dtype=torch.float64)
    with pytest.raises(ValueError, match="adjoint_precision"):
        pkg.sph_map_differentiable(pos, t, t, t, t, t, param=par, kernel=pkg.Cubic(2),
                                   adjoint_precision="fp16")
    with pytest.raises(ValueError, match="precision"):
        pkg.sph_map_differentiable(pos, t, t, t, t, t, param=par, kernel=pkg.Cubic(2),
                                   precision="fp32")


def test_kernel_constructors(pkg):
    assert pkg.WendlandC4(2).dim == 2 and pkg.Cubic().dim == 3
    assert pkg.kernel_from_name("wendlandc6", 3).kind == 3
    with pytest.raises(ValueError):
        pkg.Quintic(4)


def test_first_call_is_default_context():
    """Creating the default context before anything else loaded the library
    must not deadlock (fresh process; without a GPU it reports NO_DEVICE)."""
    import subprocess
    import sys
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import __graft_entry__ as g\n"
        "pkg = g.load_package()\n"
        "try:\n"
        "    pkg.default_context(0)\n"
        "    print('context')\n"
        "except pkg.SPHtoGridError as e:\n"
        "    print('status', e.status)\n" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() in ("context", "status 10")
