"""Project-written FITS I/O (host only): the byte layout of the standard and
round trips of the snapshot and output files."""
import gzip

import numpy as np
import pytest

from particles_gb300 import fitsio


def _minimal_fits(shape, bitpix, values):
    """A FITS file assembled card by card from the standard, independently of
    the writer: 80-byte cards, 2880-byte blocks, big-endian data."""
    cards = ["SIMPLE  =                    T", f"BITPIX  = {bitpix:>20d}",
             f"NAXIS   = {len(shape):>20d}"]
    cards += [f"NAXIS{i + 1:<3d}= {n:>20d}" for i, n in enumerate(shape[::-1])]
    cards += ["BSCALE  =                  2.0", "BZERO   =                 -1.0", "END"]
    hdr = "".join(c.ljust(80) for c in cards).encode()
    hdr += b" " * (-len(hdr) % 2880)
    dt = {-32: ">f4", -64: ">f8", 16: ">i2"}[bitpix]
    body = np.asarray(values).astype(dt).tobytes()
    return hdr + body + b"\0" * (-len(body) % 2880)


def test_reads_a_file_built_from_the_standard(tmp_path):
    vals = np.arange(24, dtype=np.float64).reshape(2, 3, 4)      # NAXIS1 = 4
    p = tmp_path / "a.fits"
    p.write_bytes(_minimal_fits((2, 3, 4), -64, vals))
    data, hdr = fitsio.read_image(p, with_header=True)
    assert hdr["NAXIS1"] == 4 and hdr["NAXIS3"] == 2
    assert data.shape == (2, 3, 4) and data.dtype == np.float64
    assert np.array_equal(data, vals * 2.0 - 1.0)                 # BSCALE / BZERO


def test_writer_layout_follows_the_standard(tmp_path):
    p = tmp_path / "b.fits"
    a = np.arange(6, dtype=np.float32).reshape(2, 3)
    fitsio.write_image(p, a, {"TUNIT": (0.5, "Time unit in seconds")})
    raw = p.read_bytes()
    assert len(raw) % 2880 == 0
    cards = [raw[i:i + 80].decode() for i in range(0, 2880, 80)]
    assert cards[0].startswith("SIMPLE  =") and cards[0][29] == "T"
    assert cards[1].split("=")[1].split("/")[0].strip() == "-32"
    assert cards[3].startswith("NAXIS1  =") and int(cards[3][10:30]) == 3
    assert any(c.startswith("TUNIT   =") for c in cards)
    assert any(c.rstrip() == "END" for c in cards)
    assert np.frombuffer(raw[2880:2880 + 24], ">f4").tolist() == [0, 1, 2, 3, 4, 5]


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.int32, np.int64, np.float32,
                                   np.float64])
@pytest.mark.parametrize("gz", [False, True])
def test_round_trip(tmp_path, dtype, gz):
    rng = np.random.default_rng(1)
    a = (rng.normal(0, 100, (3, 5, 7))).astype(dtype)
    p = tmp_path / ("c.fits.gz" if gz else "c.fits")
    fitsio.write_image(p, a)
    if gz:
        with gzip.open(p, "rb") as fh:
            assert fh.read(6) == b"SIMPLE"
    b = fitsio.read_image(p)
    assert b.dtype == np.dtype(dtype) and np.array_equal(a, b)


def test_snapshot_and_outputs(tmp_path):
    from particles_gb300 import fields
    uu, bb = fields.snapshot(8, db_rms=0.5, v_rms=0.1, seed=2)
    fitsio.write_fields(tmp_path / "snap", uu, bb, bitpix=-32)
    # one component compressed: the reader falls back to .fits.gz
    p = tmp_path / "snap" / "by.fits"
    with open(p, "rb") as src, gzip.open(str(p) + ".gz", "wb") as dst:
        dst.write(src.read())
    p.unlink()
    u2, b2 = fitsio.read_fields(tmp_path / "snap", uunit=2.0, bunit=0.5)
    assert u2.shape == uu.shape and u2.dtype == np.float64
    assert np.array_equal(u2, 2.0 * uu.astype(np.float32).astype(np.float64))
    assert np.array_equal(b2, 0.5 * bb.astype(np.float32).astype(np.float64))
    with pytest.raises(FileNotFoundError):
        fitsio.read_fields(tmp_path / "nowhere")
    state = np.random.default_rng(0).normal(size=(4, 3, 8))
    cnt = np.arange(12, dtype=np.int64).reshape(4, 3)
    time = np.linspace(0, 1, 3)
    fitsio.write_outputs(tmp_path / "out", cnt, time, state, tunit=0.25, temperature=1e6)
    s2, h = fitsio.read_image(tmp_path / "out" / "state.fits", with_header=True)
    assert np.array_equal(s2, state) and h["TEMP"] == 1e6 and h["NAXIS1"] == 8
    t2, h = fitsio.read_image(tmp_path / "out" / "time.fits", with_header=True)
    assert np.array_equal(t2, time) and h["TUNIT"] == 0.25
    assert np.array_equal(fitsio.read_image(tmp_path / "out" / "counter.fits"), cnt)


def test_state_writer_streams_rows_into_the_same_file(tmp_path):
    """Rows written in pieces through the memory map give a state.fits
    byte-identical to the one written at the end (write_outputs)."""
    from particles_gb300 import fitsio
    rng = np.random.default_rng(7)
    state = rng.normal(size=(37, 11, 8))
    fitsio.write_outputs(tmp_path / "whole", np.zeros((37, 3), np.int64), np.arange(11.0), state,
                         temperature=1.5e6)
    with fitsio.StateWriter(tmp_path / "state.fits", 37, 11, temperature=1.5e6) as w:
        for n0, n1 in ((0, 1), (1, 5), (5, 5), (5, 11)):
            w.write_rows(n0, n1, state[:, n0:n1])
    a = (tmp_path / "state.fits").read_bytes()
    b = (tmp_path / "whole" / "state.fits").read_bytes()
    assert a == b
    got, hdr = fitsio.read_image(tmp_path / "state.fits", with_header=True)
    assert np.array_equal(got, state) and hdr["TEMP"] == 1.5e6


def test_state_writer_checks_its_arguments(tmp_path):
    import pytest
    from particles_gb300 import fitsio
    with pytest.raises(ValueError):
        fitsio.StateWriter(tmp_path / "s.fits.gz", 2, 2)
    w = fitsio.StateWriter(tmp_path / "s.fits", 2, 3)
    with pytest.raises(ValueError):
        w.write_rows(2, 4, np.zeros((2, 2, 8)))
    with pytest.raises(ValueError):
        w.write_rows(0, 1, np.zeros((3, 1, 8)))
    w.close()
    empty = fitsio.StateWriter(tmp_path / "e.fits", 0, 3)
    empty.close()
    assert fitsio.read_image(tmp_path / "e.fits").shape == (0, 3, 8)
