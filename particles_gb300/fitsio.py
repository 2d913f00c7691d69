"""Minimal FITS image I/O for field snapshots and run outputs.

The reference reads its snapshot through cfitsio (sources/fitsio.F90:
`check_if_exists` :137-161 resolves `<datadir>/<name>.fits` or `.fits.gz`,
`get_dimensions` :173-196 and `read_field` :208-269 read one 3-D primary
image of BITPIX -32 or -64 per component) and scales them in
`initialize_fields` (sources/fields.F90:51-76): uu = uunit * (ux, uy, uz),
bb = bunit * (bx, by, bz).  The driver writes `counter.fits`, `time.fits`
(key TUNIT) and `state.fits` (key TEMP) at the end of a run
(sources/particles.F90:369-371, fitsio.F90 `write_data_*`).

This module implements the parts of the FITS standard those calls use --
one primary HDU holding an N-dimensional image, 80-character header cards
in 2880-byte blocks, big-endian data padded to 2880 bytes, BITPIX 8, 16,
32, 64, -32 and -64, optional gzip -- with numpy only.  Axis order follows
FITS: NAXIS1 varies fastest, so an image read here has numpy shape
(NAXISn, ..., NAXIS1), which is the Fortran array (NAXIS1, ..., NAXISn) in
C order -- the layout the integrator's C ABI takes.
"""
from __future__ import annotations

import gzip
from pathlib import Path

import numpy as np

BLOCK = 2880
_BITPIX = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}
_FROM_DTYPE = {np.dtype(np.uint8): 8, np.dtype(np.int16): 16, np.dtype(np.int32): 32,
               np.dtype(np.int64): 64, np.dtype(np.float32): -32, np.dtype(np.float64): -64}


def _card(key: str, value, comment: str = "") -> bytes:
    if isinstance(value, bool):
        v = "T" if value else "F"
        s = f"{key:<8}= {v:>20}"
    elif isinstance(value, (int, np.integer)):
        s = f"{key:<8}= {int(value):>20d}"
    elif isinstance(value, (float, np.floating)):
        txt = repr(float(value)).upper()
        if "E" not in txt and "." not in txt and "INF" not in txt and "NAN" not in txt:
            txt += ".0"
        s = f"{key:<8}= {txt:>20}"
    else:
        txt = "'" + str(value).replace("'", "''").ljust(8) + "'"
        s = f"{key:<8}= {txt:<20}"
    if comment:
        s += " / " + comment
    if len(s) > 80:
        raise ValueError(f"header card too long: {s!r}")
    return s.ljust(80).encode("ascii")


def _open(path, mode):
    path = Path(path)
    return gzip.open(path, mode) if path.suffix == ".gz" else open(path, mode)


def _header(shape, bitpix, keys=None) -> bytes:
    """Primary-HDU header of an image of numpy `shape`, padded to a block."""
    cards = [_card("SIMPLE", True, "conforms to FITS standard"),
             _card("BITPIX", bitpix, "array data type"),
             _card("NAXIS", len(shape), "number of array dimensions")]
    for i, n in enumerate(tuple(shape)[::-1]):
        cards.append(_card(f"NAXIS{i + 1}", int(n)))
    for k, v in (keys or {}).items():
        val, com = v if isinstance(v, tuple) else (v, "")
        cards.append(_card(k.upper(), val, com))
    cards.append(b"END".ljust(80))
    header = b"".join(cards)
    return header + b" " * (-len(header) % BLOCK)


def write_image(path, data, keys: dict | None = None, bitpix: int | None = None):
    """Write `data` as the primary image of a new FITS file (gzip for *.gz).

    The last numpy axis becomes NAXIS1.  bitpix (default: from the dtype)
    converts the data; keys are extra header cards {KEY: value or (value,
    comment)}."""
    data = np.asarray(data)
    if bitpix is None:
        if data.dtype not in _FROM_DTYPE:
            raise ValueError(f"no FITS BITPIX for dtype {data.dtype}")
        bitpix = _FROM_DTYPE[data.dtype]
    if bitpix not in _BITPIX:
        raise ValueError(f"unsupported BITPIX {bitpix}")
    header = _header(data.shape, bitpix, keys)
    body = np.ascontiguousarray(data).astype(_BITPIX[bitpix]).tobytes()
    body += b"\0" * (-len(body) % BLOCK)
    with _open(path, "wb") as fh:
        fh.write(header)
        fh.write(body)


def _parse_value(raw: str):
    raw = raw.split("/")[0].strip() if not raw.strip().startswith("'") else raw.strip()
    if raw.startswith("'"):
        end = 1
        out = []
        while end < len(raw):
            if raw[end] == "'":
                if end + 1 < len(raw) and raw[end + 1] == "'":
                    out.append("'")
                    end += 2
                    continue
                break
            out.append(raw[end])
            end += 1
        return "".join(out).rstrip()
    if raw in ("T", "F"):
        return raw == "T"
    try:
        return int(raw)
    except ValueError:
        return float(raw.replace("D", "E"))


def read_header(fh) -> dict:
    hdr = {}
    while True:
        block = fh.read(BLOCK)
        if len(block) < BLOCK:
            raise ValueError("truncated FITS header")
        for i in range(0, BLOCK, 80):
            card = block[i:i + 80].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                return hdr
            if card[8:10] == "= ":
                hdr[key] = _parse_value(card[10:])


def read_image(path, with_header: bool = False):
    """The primary image of a FITS file as a native-endian numpy array of
    shape (NAXISn, ..., NAXIS1); BZERO/BSCALE are applied when present."""
    with _open(path, "rb") as fh:
        hdr = read_header(fh)
        if hdr.get("SIMPLE") is not True:
            raise ValueError(f"{path}: not a FITS primary HDU")
        bitpix = int(hdr["BITPIX"])
        if bitpix not in _BITPIX:
            raise ValueError(f"{path}: unsupported BITPIX {bitpix}")
        shape = tuple(int(hdr[f"NAXIS{i}"]) for i in range(int(hdr["NAXIS"]), 0, -1))
        n = int(np.prod(shape)) if shape else 0
        dt = np.dtype(_BITPIX[bitpix])
        buf = fh.read(n * dt.itemsize)
        if len(buf) < n * dt.itemsize:
            raise ValueError(f"{path}: truncated data")
    data = np.frombuffer(buf, dt).reshape(shape).astype(dt.newbyteorder("="))
    if "BSCALE" in hdr or "BZERO" in hdr:
        data = data * float(hdr.get("BSCALE", 1.0)) + float(hdr.get("BZERO", 0.0))
    return (data, hdr) if with_header else data


# ---- the reference's snapshot and output files -------------------------

FIELD_NAMES = {"ux": "ux", "uy": "uy", "uz": "uz", "bx": "bx", "by": "by", "bz": "bz"}


def resolve(datadir, name) -> Path:
    """<datadir>/<name>.fits, else .fits.gz (fitsio.F90:137-161)."""
    for suffix in (".fits", ".fits.gz"):
        p = Path(datadir) / f"{name}{suffix}"
        if p.exists():
            return p
    raise FileNotFoundError(f"Data file for {name} does not exist under {datadir}")


def read_fields(datadir, uunit=1.0, bunit=1.0, names: dict | None = None):
    """The snapshot as the reference's uu, bb: arrays of shape (3, dm3, dm2,
    dm1) in float64 (fields.F90:51-76, fitsio.F90:208-269); names maps
    ux..bz to the file stems (the x-velocity-name ... parameters)."""
    names = {**FIELD_NAMES, **(names or {})}
    comps = []
    dm = None
    for key in ("ux", "uy", "uz", "bx", "by", "bz"):
        a, hdr = read_image(resolve(datadir, names[key]), with_header=True)
        if int(hdr["BITPIX"]) not in (-32, -64) or a.ndim != 3:
            raise ValueError(f"{names[key]}: expected a 3-D BITPIX -32/-64 image")
        if dm is None:
            dm = a.shape
        elif a.shape != dm:
            raise ValueError(f"{names[key]}: dimensions {a.shape} differ from {dm}")
        comps.append(a.astype(np.float64))
    uu = float(uunit) * np.stack(comps[:3])
    bb = float(bunit) * np.stack(comps[3:])
    return uu, bb


def write_fields(datadir, uu, bb, bitpix=-64, names: dict | None = None):
    """Write a snapshot as six 3-D images <datadir>/<name>.fits.

    BITPIX -64 (the default) keeps every bit and is read back exactly by
    read_fields.  Files meant for the reference's Fortran driver need
    bitpix=-32: its read_field reads a -64 image with the single-precision
    ftgpve into a double buffer (fitsio.F90:258-261) and so misreads it."""
    names = {**FIELD_NAMES, **(names or {})}
    Path(datadir).mkdir(parents=True, exist_ok=True)
    for i, key in enumerate(("ux", "uy", "uz")):
        write_image(Path(datadir) / f"{names[key]}.fits", uu[i], bitpix=bitpix)
    for i, key in enumerate(("bx", "by", "bz")):
        write_image(Path(datadir) / f"{names[key]}.fits", bb[i], bitpix=bitpix)


def _temp_key(temperature):
    return ({"TEMP": (float(temperature), "Initial thermal temperature")}
            if temperature is not None else None)


class StateWriter:
    """state.fits written while a run produces it (the output of
    particles.F90:371 / fitsio.F90:490-540, streamed): the header and a
    zero-filled data section are laid down once, then ranges of output rows
    are stored in place through a memory map of the big-endian data (FITS
    order: NAXIS1 = 8 fastest, NAXIS2 = m, NAXIS3 = np), so rows reach the
    file as windows finish instead of at the end.  close() flushes; the
    finished file is byte-identical to write_outputs' state.fits.  Plain
    .fits only (a gzip stream cannot be written in place)."""

    def __init__(self, path, npart: int, m: int, temperature=None):
        self.path = Path(path)
        if self.path.suffix == ".gz":
            raise ValueError("StateWriter writes plain .fits files")
        self.shape = (int(npart), int(m), 8)
        header = _header(self.shape, -64, _temp_key(temperature))
        nbytes = int(np.prod(self.shape)) * 8
        with open(self.path, "wb") as fh:
            fh.write(header)
            fh.truncate(len(header) + nbytes + (-nbytes % BLOCK))
        self._mm = np.memmap(self.path, dtype=">f8", mode="r+", offset=len(header),
                             shape=self.shape) if nbytes else None

    def write_rows(self, n0: int, n1: int, rows):
        """Store rows n0..n1-1 of every particle: rows has shape (np, n1-n0, 8)."""
        if not 0 <= n0 <= n1 <= self.shape[1]:
            raise ValueError(f"rows {n0}:{n1} outside 0:{self.shape[1]}")
        rows = np.asarray(rows, np.float64)
        if rows.shape != (self.shape[0], n1 - n0, 8):
            raise ValueError(f"rows of shape {rows.shape}, expected {(self.shape[0], n1 - n0, 8)}")
        if self._mm is not None and n1 > n0:
            self._mm[:, n0:n1, :] = rows

    def close(self):
        if self._mm is not None:
            self._mm.flush()
            self._mm = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def write_outputs(outdir, counter, time, state, tunit=None, temperature=None):
    """counter.fits (int64, NAXIS1 = 3), time.fits (key TUNIT) and state.fits
    (key TEMP, NAXIS1 = 8, NAXIS2 = m) as particles.F90:369-371 writes them."""
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    write_image(out / "counter.fits", np.asarray(counter, np.int64))
    write_image(out / "time.fits", np.asarray(time, np.float64),
                {"TUNIT": (float(tunit), "Time unit in seconds")} if tunit is not None else None)
    write_image(out / "state.fits", np.asarray(state, np.float64), _temp_key(temperature))
