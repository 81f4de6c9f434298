"""Output formats of a map: FITS images with the mapping header and VTK
rectilinear grids (SPHtoGrid.jl src/shared/io.jl:12-155,
src/shared/vtk.jl:10-21, src/shared/reconstruct_grid.jl:6-46).

Host-side code: images on the GPU are copied to the host first.  The FITS
writer emits the standard layout itself (80-character cards in 2880-byte
blocks, big-endian Float64 data with NAXIS1 the fastest axis, i.e. the
Julia column-major order of the reference's arrays); one HDU per image
``image[:, :, k]``, each carrying the reference's header keys.  The VTK
writer emits an XML RectilinearGrid (``.vtr``) with raw appended data.
"""
from __future__ import annotations

import struct

import numpy as np

from .parameters import MappingParameters, mappingParameters

_BLOCK = 2880

# header keys and comments of write_fits_image (io.jl:19-48)
_KEYS = [("SNAP", "snapshot number"),
         ("CENTER_X", "image center (x)"), ("CENTER_Y", "image center (y)"),
         ("CENTER_Z", "image center (z)"),
         ("XMIN", "x limit left"), ("XMAX", "x limit right"),
         ("YMIN", "y limit left"), ("YMAX", "y limit right"),
         ("ZMIN", "z limit left"), ("ZMAX", "z limit right"),
         ("BOXSIZE", "size of the image"), ("Z_SLICE", "depth of the integrated slice"),
         ("NPIXELS", "image resolution"), ("PIX_SIZE", "pixel size"),
         ("UNITS", "units of the image")]


def _to_host(image):
    if hasattr(image, "detach"):  # torch tensor (host or device)
        image = image.detach().cpu().numpy()
    return np.asarray(image, dtype=np.float64)


def _fmt_value(v) -> str:
    if isinstance(v, (bool, np.bool_)):
        return f"{'T' if v else 'F':>20}"
    if isinstance(v, (int, np.integer)):
        return f"{int(v):>20d}"
    if isinstance(v, (float, np.floating)):
        s = repr(float(v)).upper()
        if "INF" in s or "NAN" in s:
            raise ValueError("FITS header values must be finite")
        if "." not in s and "E" not in s:
            s += ".0"
        return f"{s:>20}"
    s = str(v).replace("'", "''")
    return f"'{s:<8}'"


def _card(key: str, value=None, comment: str = "") -> bytes:
    if key == "END":
        text = "END"
    else:
        text = f"{key:<8}= {_fmt_value(value)}"
        if comment:
            text += f" / {comment}"
    if len(text) > 80:
        text = text[:80]
    return text.ljust(80).encode("ascii")


def _pad(b: bytes, fill: bytes) -> bytes:
    r = len(b) % _BLOCK
    return b if r == 0 else b + fill * (_BLOCK - r)


def _header_values(par: MappingParameters, units: str, snap: int):
    z_slice = abs(par.z_lim[0]) + abs(par.z_lim[1])  # io.jl:17
    return [int(snap), *[float(c) for c in par.center], float(par.x_lim[0]), float(par.x_lim[1]),
            float(par.y_lim[0]), float(par.y_lim[1]), float(par.z_lim[0]), float(par.z_lim[1]),
            float(par.boxsize), float(z_slice), int(max(par.Npixels)), float(par.pixelSideLength),
            str(units)]


def write_fits_image(filename: str, image, par: MappingParameters | None = None, *,
                     units: str = "[i.u.]", snap: int = 0) -> None:
    """Write ``image`` ((P, P) or (P, P, N): one HDU per ``image[:, :, k]``)
    with the mapping parameters in every header (io.jl:12-58); without
    ``par`` only SNAP and UNITS are written (the all-sky variant,
    io.jl:67-89)."""
    img = _to_host(image)
    if img.ndim == 2:
        img = img[:, :, None]
    if img.ndim != 3:
        raise ValueError("image must be 2D or a stack of 2D images")
    if par is None:
        keys = [("SNAP", int(snap), "snapshot number"), ("UNITS", str(units), "units of the image")]
    else:
        keys = [(k, v, c) for (k, c), v in zip(_KEYS, _header_values(par, units, snap))]
    with open(filename, "wb") as f:
        for k in range(img.shape[2]):
            plane = img[:, :, k]
            cards = [_card("SIMPLE", True, "file conforms to FITS standard")] if k == 0 else \
                [_card("XTENSION", "IMAGE", "image extension")]
            cards += [_card("BITPIX", -64, "IEEE double precision"), _card("NAXIS", 2),
                      _card("NAXIS1", plane.shape[0]), _card("NAXIS2", plane.shape[1])]
            cards += [_card("EXTEND", True)] if k == 0 else \
                [_card("PCOUNT", 0), _card("GCOUNT", 1)]
            cards += [_card(key, v, c) for key, v, c in keys]
            cards.append(_card("END"))
            f.write(_pad(b"".join(cards), b" "))
            f.write(_pad(plane.astype(">f8").tobytes(order="F"), b"\0"))


def _parse_value(s: str):
    s = s.strip()
    if s.startswith("'"):
        end = s.find("'", 1)
        while end != -1 and end + 1 < len(s) and s[end + 1] == "'":
            end = s.find("'", end + 2)
        return s[1:end].replace("''", "'").rstrip()
    v = s.split("/")[0].strip()
    if v in ("T", "F"):
        return v == "T"
    try:
        return int(v)
    except ValueError:
        return float(v)


def _read_hdus(filename: str):
    with open(filename, "rb") as f:
        data = f.read()
    pos, hdus = 0, []
    while pos < len(data):
        hdr = {}
        while True:
            block = data[pos:pos + _BLOCK]
            if len(block) < _BLOCK:
                raise ValueError("truncated FITS header")
            pos += _BLOCK
            done = False
            for i in range(0, _BLOCK, 80):
                card = block[i:i + 80].decode("ascii")
                key = card[:8].strip()
                if key == "END":
                    done = True
                    break
                if card[8:10] == "= ":
                    hdr[key] = _parse_value(card[10:])
            if done:
                break
        shape = tuple(hdr.get(f"NAXIS{i + 1}", 0) for i in range(hdr.get("NAXIS", 0)))
        nbytes = int(np.prod(shape)) * abs(hdr["BITPIX"]) // 8 if shape else 0
        if hdr.get("BITPIX") != -64:
            raise ValueError("only Float64 images are read")
        arr = np.frombuffer(data, dtype=">f8", count=nbytes // 8, offset=pos)
        hdus.append((hdr, arr.reshape(shape, order="F").astype(np.float64)))
        pos += nbytes + (-nbytes) % _BLOCK
    return hdus


def read_fits_image(filename: str, Nimage: int = 1):
    """(image, mappingParameters, snap, units) of HDU ``Nimage`` (1-based),
    the parameters rebuilt from the header as io.jl:132-138 does."""
    hdr, img = _read_hdus(filename)[Nimage - 1]
    par = mappingParameters(x_lim=[hdr["XMIN"], hdr["XMAX"]], y_lim=[hdr["YMIN"], hdr["YMAX"]],
                            z_lim=[hdr["ZMIN"], hdr["ZMAX"]], Npixels=int(hdr["NPIXELS"]),
                            boxsize=hdr["BOXSIZE"])
    return img, par, hdr["SNAP"], hdr["UNITS"]


def read_allsky_fits_image(filename: str):
    """(image, snap, units) of the first HDU (io.jl:158-185)."""
    hdr, img = _read_hdus(filename)[0]
    return img, hdr["SNAP"], hdr["UNITS"]


def get_map_grid_2D(par: MappingParameters):
    """Pixel-centre coordinates (reconstruct_grid.jl:6-20)."""
    psl = par.pixelSideLength
    x = par.x_lim[0] + (np.arange(1, par.Npixels[0] + 1) - 0.5) * psl
    y = par.y_lim[0] + (np.arange(1, par.Npixels[1] + 1) - 0.5) * psl
    return x, y


def get_map_grid_3D(par: MappingParameters):
    """Pixel-centre coordinates (reconstruct_grid.jl:27-46).  The reference
    offsets the z grid by y_lim[1] rather than z_lim[1] (:42); kept, so the
    grids written here are the reference's."""
    x, y = get_map_grid_2D(par)
    z = par.y_lim[0] + (np.arange(1, par.Npixels[2] + 1) - 0.5) * par.pixelSideLength
    return x, y, z


def write_vtk_image(filename: str, image, image_name: str, par: MappingParameters, *,
                    units: str = "[i.u.]", snap: int = 0) -> str:
    """A 3D map as a VTK XML RectilinearGrid on the pixel centres, the image
    as point data in its array order (first index fastest), Units and Snap
    as field data (vtk.jl:10-21).  Returns the file name written (``.vtr``
    appended when missing)."""
    img = _to_host(image)
    if img.ndim != 3:
        raise ValueError("write_vtk_image takes a 3D map")
    if not filename.endswith(".vtr"):
        filename += ".vtr"
    x, y, z = get_map_grid_3D(par)
    nx, ny, nz = img.shape
    if (len(x), len(y), len(z)) != (nx, ny, nz):
        raise ValueError("image shape does not match the mapping parameters")
    arrays = [img.astype("<f8").tobytes(order="F"), np.asarray(x, "<f8").tobytes(),
              np.asarray(y, "<f8").tobytes(), np.asarray(z, "<f8").tobytes()]
    offs, o = [], 0
    for a in arrays:
        offs.append(o)
        o += 8 + len(a)
    ext = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    units_xml = str(units).replace("&", "&amp;").replace("<", "&lt;").replace(">", "&gt;")
    name_xml = str(image_name).replace("&", "&amp;").replace('"', "&quot;").replace("<", "&lt;")
    head = (
        '<?xml version="1.0"?>\n'
        '<VTKFile type="RectilinearGrid" version="1.0" byte_order="LittleEndian" '
        'header_type="UInt64">\n'
        f'  <RectilinearGrid WholeExtent="{ext}">\n'
        '    <FieldData>\n'
        f'      <Array type="String" Name="Units" NumberOfTuples="1" format="ascii">'
        f'{units_xml}</Array>\n'
        f'      <DataArray type="Int64" Name="Snap" NumberOfTuples="1" format="ascii">'
        f'{int(snap)}</DataArray>\n'
        '    </FieldData>\n'
        f'    <Piece Extent="{ext}">\n'
        f'      <PointData Scalars="{name_xml}">\n'
        f'        <DataArray type="Float64" Name="{name_xml}" format="appended" offset="{offs[0]}"/>\n'
        '      </PointData>\n'
        '      <Coordinates>\n'
        f'        <DataArray type="Float64" Name="x" format="appended" offset="{offs[1]}"/>\n'
        f'        <DataArray type="Float64" Name="y" format="appended" offset="{offs[2]}"/>\n'
        f'        <DataArray type="Float64" Name="z" format="appended" offset="{offs[3]}"/>\n'
        '      </Coordinates>\n'
        '    </Piece>\n'
        '  </RectilinearGrid>\n'
        '  <AppendedData encoding="raw">\n_')
    with open(filename, "wb") as f:
        f.write(head.encode("utf-8"))
        for a in arrays:
            f.write(struct.pack("<Q", len(a)))
            f.write(a)
        f.write(b"\n  </AppendedData>\n</VTKFile>\n")
    return filename
