"""The C++ drop-in on the CPU: a program that includes include/El_gb300.hpp
in place of Elemental's El.hpp compiles with g++, links libelgb300.so and runs
the path's host-side pieces with the reference's semantics -- El::Matrix
(owned, copied, moved, attached, and views A(IR, IR) / El::View with END,
include/El/core/View/impl.hpp:274-387, also through ElView_d), El::Permutation swap sequences with implicit
and explicit origins (src/lapack_like/perm/Permutation.cpp:205-303, 436-450,
544-631, 731-745) and their implicit-origin form for the device, the
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
#include "El_gb300.h"
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
  // explicit origins from the first swap whose origin is not the swap count
  Permutation E;
  E.MakeIdentity(4);
  E.Swap(2, 0);
  E.Swap(3, 1);
  E.Swap(1, 1);
  if (E.IsImplicitSwapSequence()) return 12;
  const Matrix<Int> eo = E.SwapOrigins();
  if (eo.Height() != 3 || eo.Get(0, 0) != 2 || eo.Get(1, 0) != 3 || eo.Get(2, 0) != 1)
    return 13;
  if (E.Parity()) return 14;  // two non-trivial swaps
  Matrix<Int> e;
  E.ExplicitVector(e);  // [0 1 2 3] -> [2 1 0 3] -> [2 3 0 1]
  if (e.Get(0, 0) != 2 || e.Get(1, 0) != 3 || e.Get(2, 0) != 0 || e.Get(3, 0) != 1) return 15;
  // the implicit-origin sequence handed to the device replays the same rows
  const std::vector<Int> di = E.ImplicitSwapDests(4);
  Permutation I;
  I.SetSwapSequence(4, di.data(), 4);
  Matrix<Int> ie;
  I.ExplicitVector(ie);
  for (Int k = 0; k < 4; ++k)
    if (ie.Get(k, 0) != e.Get(k, 0)) return 16;
  Matrix<double> M(4, 1);
  for (Int i = 0; i < 4; ++i) M.Set(i, 0, i);
  E.PermuteRows(M);
  for (Int i = 0; i < 4; ++i)
    if (M.Get(i, 0) != e.Get(i, 0)) return 17;
  E.InversePermuteRows(M);
  for (Int i = 0; i < 4; ++i)
    if (M.Get(i, 0) != i) return 18;
  // appending another sequence with an offset, and appending to itself
  Permutation F;
  F.MakeIdentity(6);
  F.SwapSequence(E, 2);
  if (F.NumSwaps() != 3 || F.SwapOrigins().Get(0, 0) != 4 || F.SwapDestinations().Get(0, 0) != 2)
    return 19;
  F.SwapSequence(F);
  if (F.NumSwaps() != 6) return 20;
  Permutation G;
  G.MakeIdentity(3);
  Matrix<Int> gd(2, 1);
  gd.Set(0, 0, 2);
  gd.Set(1, 0, 1);
  G.ImplicitSwapSequence(gd);
  if (!G.IsImplicitSwapSequence() || G.NumSwaps() != 2) return 21;
  // random explicit-origin sequences: the implicit form permutes identically
  unsigned long long seed = 12345;
  auto next = [&seed](Int m) {
    seed = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    return (Int)((seed >> 33) % (unsigned long long)m);
  };
  for (int trial = 0; trial < 200; ++trial) {
    const Int n = 1 + next(12);
    Permutation R2;
    R2.MakeIdentity(n);
    const Int swaps = next(2 * n + 1);
    for (Int k = 0; k < swaps; ++k) R2.Swap(next(n), next(n));
    Matrix<Int> r, ri;
    R2.ExplicitVector(r);
    const std::vector<Int> d2 = R2.ImplicitSwapDests(n);
    Permutation I2;
    I2.SetSwapSequence(n, d2.data(), n);
    I2.ExplicitVector(ri);
    for (Int k = 0; k < n; ++k) {
      if (ri.Get(k, 0) != r.Get(k, 0)) return 22;
      if (!R2.IsImplicitSwapSequence() && d2[k] < k) return 23;  // rewritten: dest >= k
    }
  }
  // views: A(IR, IR) shares A's buffer; END resolves to the extent
  Matrix<double> W(5, 4);
  for (Int j = 0; j < 4; ++j)
    for (Int i = 0; i < 5; ++i) W.Set(i, j, 100.0 * i + j);
  auto S = W(IR(1, 4), IR(2, END));
  if (!S.Viewing() || S.Height() != 3 || S.Width() != 2 || S.LDim() != 5) return 24;
  if (S.Get(0, 0) != 102.0 || S.Get(2, 1) != 303.0) return 25;
  S.Set(1, 1, -1.0);
  if (W.Get(2, 3) != -1.0) return 26;
  const Matrix<double>& Wc = W;
  auto L = Wc(ALL, IR(1));
  if (!L.Locked() || L.Height() != 5 || L.Width() != 1 || L.Get(4, 0) != 401.0) return 27;
  try {
    L.Buffer();
    return 28;
  } catch (const std::logic_error&) {
  }
  try {
    W(IR(0, 6), ALL);
    return 29;
  } catch (const std::logic_error&) {
  }
  Matrix<double> X2;
  View(X2, W, 1, 1, 2, 2);
  if (X2.Get(1, 1) != 202.0) return 30;
  // a permutation applied through a view moves the parent's rows
  Permutation Q2;
  Q2.MakeIdentity(3);
  Q2.Swap(0, 2);
  Q2.PermuteRows(S);
  if (W.Get(1, 2) != 302.0 || W.Get(3, 2) != 102.0 || W.Get(1, 1) != 101.0) return 31;
  // moving keeps an owned matrix's data; copying a view gives an owned copy
  Matrix<double> Mv(std::move(C));
  if (Mv.Get(2, 1) != 12.0 || C.Height() != 0) return 32;
  Matrix<double> Cp(S);
  if (Cp.Viewing() || Cp.Get(1, 1) != -1.0) return 33;
  // the same through the C interface
  ElMatrix_d cA, cV;
  ElMatrixCreate_d(&cA);
  ElMatrixCreate_d(&cV);
  ElMatrixResize_d(cA, 4, 3);
  ElMatrixSet_d(cA, 2, 1, 5.0);
  ElRange_i ri = {1, 3}, rj = {0, -100};
  if (ElView_d(cV, cA, ri, rj) != EL_SUCCESS) return 34;
  double v = 0;
  ElInt h = 0;
  ElMatrixGet_d(cV, 1, 1, &v);
  ElMatrixHeight_d(cV, &h);
  if (v != 5.0 || h != 2) return 35;
  ElRange_i bad = {0, 9};
  if (ElView_d(cV, cA, bad, rj) != EL_LOGIC_ERROR) return 36;
  ElMatrixDestroy_d(cV);
  ElMatrixDestroy_d(cA);
  // the header's inline solver entry points instantiate for the path's types
  void (*hpd_d)(UpperOrLower, Orientation, Matrix<double>&, Matrix<double>&) =
      &hpd_solve::Overwrite<double>;
  void (*hpd_s)(UpperOrLower, Orientation, Matrix<float>&, Matrix<float>&) =
      &hpd_solve::Overwrite<float>;
  if (!hpd_d || !hpd_s) return 37;
  // copying into a proper sub-view writes the parent's entries in place
  // (the view keeps its leading dimension, include/El/core/Matrix/impl.hpp:698-716)
  Matrix<double> Pm(4, 4);
  for (Int j = 0; j < 4; ++j)
    for (Int i = 0; i < 4; ++i) Pm.Set(i, j, 10.0 * i + j);
  Matrix<double> Sm(2, 2);
  Sm.Set(0, 0, -1.0);
  Sm.Set(1, 0, -2.0);
  Sm.Set(0, 1, -3.0);
  Sm.Set(1, 1, -4.0);
  auto Vw = Pm(IR(1, 3), IR(2, 4));
  Vw = Sm;
  if (!Vw.Viewing() || Vw.LDim() != 4) return 38;
  if (Pm.Get(1, 2) != -1.0 || Pm.Get(2, 2) != -2.0 || Pm.Get(1, 3) != -3.0 ||
      Pm.Get(2, 3) != -4.0 || Pm.Get(0, 2) != 2.0 || Pm.Get(3, 3) != 33.0)
    return 39;
  // moving into a view copies the entries too
  Matrix<double> Sm2(Sm);
  Sm2.Set(0, 0, 99.0);
  Vw = std::move(Sm2);
  if (Pm.Get(1, 2) != 99.0) return 40;
  // a view may shrink but not grow
  auto Vw2 = Pm(IR(0, 2), ALL);
  Vw2.Resize(2, 4);
  Vw2.Resize(1, 3);
  if (Vw2.LDim() != 4 || Vw2.Height() != 1 || Vw2.Width() != 3) return 41;
  try {
    Vw2.Resize(3, 3);
    return 42;
  } catch (const std::logic_error&) {
  }
  // copying into a locked view raises the reference's LogicError
  Matrix<double> Lk;
  LockedView(Lk, Pm, 0, 0, 2, 2);
  try {
    Lk = Sm;
    return 43;
  } catch (const std::logic_error&) {
  }
  if (Pm.Get(0, 0) != 0.0 || Pm.Get(1, 1) != 11.0) return 44;
  // shrinking an owned matrix keeps its buffer, leading dimension and entries
  Pm.Resize(2, 3);
  if (Pm.LDim() != 4 || Pm.Get(1, 2) != 99.0 || Pm.Get(0, 1) != 1.0) return 45;
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


C_PROGRAM = r"""
#include "El_gb300.h"
#include <stdio.h>

int main(void) {
  ElMatrix_d A, V;
  ElPermutation P;
  ElRange_i rows = {1, 3}, cols = {0, -100};
  double v = 0.0;
  ElInt h = 0, nb = 0;
  if (ElMatrixCreate_d(&A) != EL_SUCCESS || ElMatrixCreate_d(&V) != EL_SUCCESS) return 1;
  if (ElMatrixResize_d(A, 4, 2) != EL_SUCCESS) return 2;
  ElMatrixSet_d(A, 2, 1, 3.5);
  if (ElView_d(V, A, rows, cols) != EL_SUCCESS) return 3;
  ElMatrixGet_d(V, 1, 1, &v);
  ElMatrixHeight_d(V, &h);
  if (v != 3.5 || h != 2) return 4;
  if (ElPermutationCreate(&P) != EL_SUCCESS) return 5;
  ElPermutationMakeIdentity(P, 2);
  ElPermutationSwap(P, 0, 1);
  if (ElPermutationPermuteRows_d(P, V, 0) != EL_SUCCESS) return 6;
  ElMatrixGet_d(A, 1, 1, &v);
  if (v != 3.5) return 7;
  if (ElPermutationSwap(P, 0, 9) != EL_LOGIC_ERROR) return 8;
  ElBlocksize(&nb);
  if (nb != 128) return 9;
  ElPermutationDestroy(P);
  ElMatrixDestroy_d(V);
  ElMatrixDestroy_d(A);
  puts("c ok");
  return 0;
}
"""


@pytest.mark.parametrize("std", ["c99", "c11"])
def test_c_program_builds_against_the_c_interface_and_runs(tmp_path, std):
    """include/El_gb300.h is plain C (a C caller of Elemental's interface):
    it compiles warning-free as C99 (the reference's C headers need C99 too:
    stdbool.h, long long) and C11, and the host-side entry points behave as
    the reference's."""
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    assert os.path.exists(LIB), "libelgb300.so not built"
    src = tmp_path / "cabi.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "cabi"
    r = subprocess.run([gcc, f"-std={std}", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src), "-L", LIBDIR, "-lelgb300",
                        "-Wl,-rpath," + LIBDIR, "-o", str(exe)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0 and run.stdout.strip() == "c ok", (run.returncode, run.stdout)
