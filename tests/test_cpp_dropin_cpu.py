"""The C++ drop-in on the CPU: a program that includes include/El_gb300.hpp
in place of Elemental's El.hpp compiles with g++, links libelgb300.so and runs
the path's host-side pieces with the reference's semantics -- El::Matrix
(owned, copied, attached views), El::Permutation swap sequences
(src/lapack_like/perm/Permutation.cpp:205-250, 544-631, 731-745), the
blocksize stack (src/blas_like/blocksizes.cpp:37-60) and El::Write / El::Read
(src/io/Write/Binary.hpp:17-37, src/io/Read/Binary.hpp:17-44).  No GPU
call."""
import os
import shutil
import subprocess

import pytest

from elemental_gb300.build import LIB, LIBDIR

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "El_gb300.hpp"
#include <cstdio>
#include <string>

int main(int argc, char** argv) {
  using namespace El;
  if (argc < 2) return 100;
  Matrix<double> A(3, 2);
  for (Int j = 0; j < 2; ++j)
    for (Int i = 0; i < 3; ++i) A.Set(i, j, i + 10.0 * j);
  // an attached view writes through to the caller's buffer (LDim 4)
  double buf[8] = {0};
  Matrix<double> V;
  V.Attach(2, 2, buf, 4);
  V.Set(1, 1, 7.0);
  if (buf[5] != 7.0 || !V.Viewing() || V.LDim() != 4) return 1;
  // a copy owns its data
  Matrix<double> C(A);
  if (C.Get(2, 1) != 12.0 || C.Viewing()) return 2;
  // swaps (0, 2) then (1, 2): rows [2, 0, 1] of the original
  Permutation P;
  P.MakeIdentity(3);
  P.ReserveSwaps(3);
  P.Swap(0, 2);
  P.Swap(1, 2);
  Matrix<Int> p;
  P.ExplicitVector(p);
  if (p.Get(0, 0) != 2 || p.Get(1, 0) != 0 || p.Get(2, 0) != 1) return 3;
  Matrix<double> B(A);
  P.PermuteRows(B);
  for (Int j = 0; j < 2; ++j)
    for (Int i = 0; i < 3; ++i)
      if (B.Get(i, j) != A.Get(p.Get(i, 0), j)) return 4;
  P.InversePermuteRows(B);
  for (Int j = 0; j < 2; ++j)
    for (Int i = 0; i < 3; ++i)
      if (B.Get(i, j) != A.Get(i, j)) return 5;
  const Matrix<Int> d = P.SwapDestinations();
  if (d.Height() != 2 || d.Get(0, 0) != 2 || d.Get(1, 0) != 2) return 6;
  // the blocksize stack
  if (Blocksize() != 128) return 7;
  PushBlocksizeStack(96);
  if (Blocksize() != 96) return 8;
  PopBlocksizeStack();
  if (Blocksize() != 128) return 9;
  // file round trip, format picked from the extension
  const std::string base = argv[1];
  Write(A, base, BINARY);
  Matrix<double> R;
  Read(R, base + ".bin");
  if (R.Height() != 3 || R.Width() != 2 || R.Get(2, 1) != 12.0) return 10;
  try {
    Read(R, base + ".xyz");
    return 11;
  } catch (const std::runtime_error&) {
  }
  std::puts("dropin ok");
  return 0;
}
"""


def test_cpp_program_builds_against_the_dropin_header_and_runs(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    assert os.path.exists(LIB), "libelgb300.so not built"
    src = tmp_path / "dropin.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", LIBDIR, "-lelgb300", "-Wl,-rpath," + LIBDIR, "-o", str(exe)],
                   check=True, capture_output=True, text=True, timeout=300)
    r = subprocess.run([str(exe), str(tmp_path / "m")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.strip() == "dropin ok"
    # the file is the reference's BINARY layout: Int height, Int width, entries
    raw = (tmp_path / "m.bin").read_bytes()
    assert len(raw) == 2 * 4 + 6 * 8
