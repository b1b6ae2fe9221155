"""El::Read / El::Write on host matrices (no GPU involved), against the bytes
the reference's own El::Write produced (tests/golden/io_write_*.npz, made by
tests/golden/gen_golden.py from the compiled reference): BINARY = [Int
height][Int width][column-major entries] in basename.bin, BINARY_FLAT = the
entries only in basename.dat (src/io/Write/Binary.hpp:17-37,
src/io/Read/Binary.hpp:17-44, src/io/File.cpp:28-70)."""
import os

import numpy as np
import pytest

import elemental_gb300 as El

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


@pytest.mark.parametrize("fmt", ["bin", "dat"])
@pytest.mark.parametrize("sfx", ["d", "s"])
def test_write_is_byte_identical_to_reference(tmp_path, fmt, sfx):
    g = load(f"io_write_{fmt}_{sfx}_7x5")
    A = El.Matrix(g["A"].copy(order="F"))
    base = str(tmp_path / "m")
    El.Write(A, base, El.BINARY if fmt == "bin" else El.BINARY_FLAT)
    with open(base + "." + fmt, "rb") as f:
        assert f.read() == bytes(g["raw"])


@pytest.mark.parametrize("sfx", ["d", "s"])
def test_read_reference_files(tmp_path, sfx):
    g = load(f"io_write_bin_{sfx}_7x5")
    path = tmp_path / "ref.bin"
    path.write_bytes(bytes(g["raw"]))
    A = El.Matrix(np.zeros((1, 1), dtype=g["A"].dtype))
    El.Read(A, str(path))  # AUTO: .bin -> BINARY, resizes to 7 x 5
    assert A.array.shape == (7, 5) and np.array_equal(A.array, g["A"])
    gf = load(f"io_write_dat_{sfx}_7x5")
    pf = tmp_path / "ref.dat"
    pf.write_bytes(bytes(gf["raw"]))
    B = El.Matrix(np.zeros((7, 5), dtype=gf["A"].dtype, order="F"))
    El.Read(B, str(pf))  # BINARY_FLAT into B's current 7 x 5 shape
    assert np.array_equal(B.array, gf["A"])


def test_int_round_trip_and_edges(tmp_path):
    M = np.arange(12, dtype=np.int32).reshape(3, 4)
    A = El.Matrix(M.copy(order="F"))
    El.Write(A, str(tmp_path / "i"))  # default BINARY
    B = El.Matrix(np.zeros((1, 1), dtype=np.int32))
    El.Read(B, str(tmp_path / "i.bin"), El.BINARY)
    assert np.array_equal(B.array, M)
    E = El.Matrix(np.zeros((0, 0)))  # empty matrix
    El.Write(E, str(tmp_path / "e"))
    assert (tmp_path / "e.bin").stat().st_size == 8
    F = El.Matrix(np.ones((2, 2)))
    El.Read(F, str(tmp_path / "e.bin"))
    assert F.array.shape == (0, 0)


def test_read_errors(tmp_path):
    A = El.Matrix(np.zeros((2, 2)))
    with pytest.raises(El.ElError):  # missing file
        El.Read(A, str(tmp_path / "missing.bin"))
    bad = tmp_path / "short.bin"
    bad.write_bytes(np.array([3, 3], dtype=np.int32).tobytes() + b"\0" * 8)
    with pytest.raises(El.ElError):  # size does not match the header
        El.Read(A, str(bad))
    with pytest.raises(El.ElError):  # ASCII is not on this path (logic error)
        El.Read(A, str(bad), El.ASCII)
    with pytest.raises(El.ElError):
        El.Write(A, str(tmp_path / "x"), El.MATRIX_MARKET)
    odd = tmp_path / "m.unknown"
    odd.write_bytes(b"")
    with pytest.raises(El.ElError):  # AUTO cannot detect the format
        El.Read(A, str(odd))
