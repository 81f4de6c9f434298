"""Output formats (io.jl, vtk.jl, reconstruct_grid.jl): FITS round trip as
the reference's own test does (runtests.jl:466-474), the FITS block layout,
the VTK rectilinear grid and the pixel-centre grids."""
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest


@pytest.fixture
def par(pkg):
    return pkg.mappingParameters(center=[3.0, 3.0, 3.0], x_size=6.0, y_size=6.0, z_size=6.0,
                                 Npixels=20, boxsize=6.0)


def test_fits_round_trip(pkg, par, tmp_path):
    from sphtogrid_gb300 import io
    rng = np.random.default_rng(3)
    img = rng.lognormal(size=(20, 20, 2))
    fn = str(tmp_path / "image.fits")
    io.write_fits_image(fn, img, par, units="K", snap=12)
    raw = open(fn, "rb").read()
    assert len(raw) % 2880 == 0
    assert raw[:30] == b"SIMPLE  =                    T"
    for k in (1, 2):
        got, fpar, snap, units = io.read_fits_image(fn, k)
        assert np.array_equal(got, img[:, :, k - 1])
        assert fpar.boxsize == par.boxsize and fpar.center == par.center
        assert fpar.x_lim == par.x_lim and fpar.Npixels == par.Npixels
        assert snap == 12 and units == "K"


def test_fits_header_keys(pkg, par, tmp_path):
    from sphtogrid_gb300 import io
    fn = str(tmp_path / "image.fits")
    io.write_fits_image(fn, np.zeros((20, 20)), par)
    hdr, data = io._read_hdus(fn)[0]
    keys = ["SNAP", "CENTER_X", "CENTER_Y", "CENTER_Z", "XMIN", "XMAX", "YMIN", "YMAX", "ZMIN",
            "ZMAX", "BOXSIZE", "Z_SLICE", "NPIXELS", "PIX_SIZE", "UNITS"]
    assert all(k in hdr for k in keys)
    assert hdr["Z_SLICE"] == abs(par.z_lim[0]) + abs(par.z_lim[1])
    assert hdr["NPIXELS"] == 20 and hdr["PIX_SIZE"] == par.pixelSideLength
    assert hdr["UNITS"] == "[i.u.]" and hdr["BITPIX"] == -64
    # data: big-endian Float64, NAXIS1 fastest, right after the header blocks
    assert data.shape == (20, 20)


def test_fits_column_major(pkg, par, tmp_path):
    from sphtogrid_gb300 import io
    img = np.arange(400, dtype=np.float64).reshape(20, 20, order="F")
    fn = str(tmp_path / "c.fits")
    io.write_fits_image(fn, img, par)
    raw = open(fn, "rb").read()
    first = struct.unpack(">2d", raw[2880:2896])
    assert first == (0.0, 1.0)  # img[0,0], img[1,0]: first index fastest


def test_allsky_fits(pkg, tmp_path):
    from sphtogrid_gb300 import io
    img = np.linspace(0, 1, 48).reshape(6, 8)
    fn = str(tmp_path / "allsky.fits")
    io.write_fits_image(fn, img, units="mJy", snap=3)
    got, snap, units = io.read_allsky_fits_image(fn)
    assert np.array_equal(got, img) and snap == 3 and units == "mJy"


def test_map_grids(pkg, par):
    from sphtogrid_gb300 import io
    x, y = io.get_map_grid_2D(par)
    assert len(x) == 20 and x[0] == par.x_lim[0] + 0.5 * par.pixelSideLength
    x3, y3, z3 = io.get_map_grid_3D(par)
    assert np.array_equal(z3, par.y_lim[0] + (np.arange(1, 21) - 0.5) * par.pixelSideLength)


def test_vtk_rectilinear_grid(pkg, par, tmp_path):
    from sphtogrid_gb300 import io
    rng = np.random.default_rng(5)
    img = rng.random((20, 20, 20))
    fn = io.write_vtk_image(str(tmp_path / "map"), img, "map", par, units="g/cm^3", snap=7)
    raw = open(fn, "rb").read()
    cut = raw.index(b"<AppendedData")
    head = raw[:cut].decode() + "</VTKFile>"
    root = ET.fromstring(head.replace("<AppendedData", ""))
    grid = root.find("RectilinearGrid")
    assert grid.get("WholeExtent") == "0 19 0 19 0 19"
    base = raw.index(b"_", cut) + 1
    arrays = {}
    for da in root.iter("DataArray"):
        if da.get("format") != "appended":
            continue
        off = base + int(da.get("offset"))
        n = struct.unpack("<Q", raw[off:off + 8])[0]
        arrays[da.get("Name")] = np.frombuffer(raw[off + 8:off + 8 + n], dtype="<f8")
    assert np.array_equal(arrays["map"], img.reshape(-1, order="F"))
    x, y, z = io.get_map_grid_3D(par)
    assert np.array_equal(arrays["x"], x) and np.array_equal(arrays["z"], z)
    field = root.find("RectilinearGrid/FieldData")
    assert field.find("Array").text == "g/cm^3"


def test_oracle_map_round_trip(pkg, oracle, tmp_path):
    """A map written and read back equals the map (runtests.jl:466-474)."""
    from sphtogrid_gb300 import io
    rng = np.random.default_rng(9)
    n = 500
    pos = np.asfortranarray(rng.uniform(0.0, 6.0, (3, n)))
    hsml = rng.uniform(0.05, 0.5, n)
    m = np.full(n, 1.0 / n)
    rho = rng.uniform(0.5, 2.0, n)
    opar = oracle.mapping_parameters(center=[3.0, 3.0, 3.0], x_size=6.0, y_size=6.0, z_size=6.0,
                                     Npixels=32, boxsize=6.0)
    img, _ = oracle.sph_mapping(pos, hsml, m, rho, rho, rho, param=opar, kernel="cubic")
    par = pkg.mappingParameters(center=[3.0, 3.0, 3.0], x_size=6.0, y_size=6.0, z_size=6.0,
                                Npixels=32, boxsize=6.0)
    fn = str(tmp_path / "map.fits")
    io.write_fits_image(fn, img, par)
    got, fpar, _, _ = io.read_fits_image(fn)
    assert np.array_equal(got, img[:, :, 0])
    assert fpar.boxsize == par.boxsize and fpar.center == par.center
