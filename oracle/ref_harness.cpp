// Command-line harness around the reference's OWN sequential factor-and-solve
// path, compiled from the reference sources by oracle/build_ref.sh.  Test
// infrastructure only (it produces the golden fixtures and validates the C
// restatement in oracle/el_oracle.c); the product never links it.
//
// Matrices travel as files in Elemental's binary layout
// ([Int height][Int width][column-major entries], src/io/Write/Binary.hpp:17-37),
// with 32-bit Int.  The harness never constructs El::Environment (that would
// initialise MPI, src/core/environment.cpp:132-198); it only pushes the
// blocksize the run asks for (src/blas_like/blocksizes.cpp:37-60).
//
//   elref <d|s> lu        <nb> A LU piv
//   elref <d|s> lusolve   <nb> <N|T> A B LU piv X
//   elref <d|s> chol      <nb> <L|U> A C
//   elref <d|s> cholpiv   <nb> <L|U> A C piv            (El::Cholesky(uplo, A, P))
//   elref <d|s> cholpivsolve <nb> <L|U> A B C piv X    (+ cholesky::SolveAfter with P)
//   elref <d|s> cholsolve <nb> <L|U> A B C X
//   elref <d|s> linsolve  <nb> A B X
//   elref <d|s> hpdsolve  <nb> <L|U> A B X
//   elref <d|s> lunopiv   <nb> A LU         (El::LU without pivoting)
//   elref <d|s> lufull    <nb> A LU p q     (El::LU with full pivoting)
//   elref <d|s> lufullsolve <nb> <N|T> A B LU p q X  (+ lu::SolveAfter with P, Q)
//   elref <d|s> inverse   <nb> A Ainv       (El::Inverse)
//   elref <d|s> onecond   <nb> A cond       (El::OneCondition, a 1 x 1 matrix)
//   elref <d|s> write     <nb> <bin|dat> basename A   (El::Write, BINARY / BINARY_FLAT)
//   elref <d|s> read      <nb> file A                 (El::Read, format from the extension)
//   elref <d|s> lutime    <nb> A reps       (prints seconds per El::LU)
// Exit status: 0 ok, 3 SingularMatrixException, 4 NonHPDMatrixException,
// 2 usage / IO error.
#include <El.hpp>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

template <typename T>
bool ReadMatrix(const char* path, El::Matrix<T>& A) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  El::Int hw[2];
  if (std::fread(hw, sizeof(El::Int), 2, f) != 2) { std::fclose(f); return false; }
  A.Resize(hw[0], hw[1]);
  for (El::Int j = 0; j < hw[1]; ++j) {
    if (hw[0] && std::fread(A.Buffer(0, j), sizeof(T), hw[0], f) != size_t(hw[0])) {
      std::fclose(f);
      return false;
    }
  }
  std::fclose(f);
  return true;
}

template <typename T>
bool WriteMatrix(const char* path, const El::Matrix<T>& A) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return false;
  El::Int hw[2] = {A.Height(), A.Width()};
  std::fwrite(hw, sizeof(El::Int), 2, f);
  for (El::Int j = 0; j < A.Width(); ++j)
    std::fwrite(A.LockedBuffer(0, j), sizeof(T), A.Height(), f);
  std::fclose(f);
  return true;
}

bool WritePivots(const char* path, const El::Permutation& P) {
  const El::Matrix<El::Int> d = P.SwapDestinations();
  return WriteMatrix(path, d);
}

El::UpperOrLower Uplo(const char* s) { return s[0] == 'U' ? El::UPPER : El::LOWER; }
El::Orientation Orient(const char* s) {
  return s[0] == 'T' ? El::TRANSPOSE : (s[0] == 'C' ? El::ADJOINT : El::NORMAL);
}

template <typename T>
int Run(int argc, char** argv) {
  const std::string op = argv[2];
  const int nb = std::atoi(argv[3]);
  El::PushBlocksizeStack(nb);
  El::Matrix<T> A, B;
  El::Permutation P;
  if (op == "lu" && argc == 7) {
    if (!ReadMatrix(argv[4], A)) return 2;
    El::LU(A, P);
    return (WriteMatrix(argv[5], A) && WritePivots(argv[6], P)) ? 0 : 2;
  }
  if (op == "lusolve" && argc == 10) {
    if (!ReadMatrix(argv[5], A) || !ReadMatrix(argv[6], B)) return 2;
    El::LU(A, P);
    El::lu::SolveAfter(Orient(argv[4]), A, P, B);
    return (WriteMatrix(argv[7], A) && WritePivots(argv[8], P) &&
            WriteMatrix(argv[9], B)) ? 0 : 2;
  }
  if (op == "chol" && argc == 7) {
    if (!ReadMatrix(argv[5], A)) return 2;
    El::Cholesky(Uplo(argv[4]), A);
    return WriteMatrix(argv[6], A) ? 0 : 2;
  }
  if (op == "cholpiv" && argc == 8) {
    if (!ReadMatrix(argv[5], A)) return 2;
    El::Cholesky(Uplo(argv[4]), A, P);
    return (WriteMatrix(argv[6], A) && WritePivots(argv[7], P)) ? 0 : 2;
  }
  if (op == "cholpivsolve" && argc == 10) {
    if (!ReadMatrix(argv[5], A) || !ReadMatrix(argv[6], B)) return 2;
    El::Cholesky(Uplo(argv[4]), A, P);
    El::cholesky::SolveAfter(Uplo(argv[4]), El::NORMAL, A, P, B);
    return (WriteMatrix(argv[7], A) && WritePivots(argv[8], P) && WriteMatrix(argv[9], B))
               ? 0 : 2;
  }
  if (op == "cholsolve" && argc == 9) {
    if (!ReadMatrix(argv[5], A) || !ReadMatrix(argv[6], B)) return 2;
    El::Cholesky(Uplo(argv[4]), A);
    El::cholesky::SolveAfter(Uplo(argv[4]), El::NORMAL, A, B);
    return (WriteMatrix(argv[7], A) && WriteMatrix(argv[8], B)) ? 0 : 2;
  }
  if (op == "linsolve" && argc == 7) {
    if (!ReadMatrix(argv[4], A) || !ReadMatrix(argv[5], B)) return 2;
    El::LinearSolve(A, B);
    return WriteMatrix(argv[6], B) ? 0 : 2;
  }
  if (op == "hpdsolve" && argc == 8) {
    if (!ReadMatrix(argv[5], A) || !ReadMatrix(argv[6], B)) return 2;
    El::HPDSolve(Uplo(argv[4]), El::NORMAL, A, B);
    return WriteMatrix(argv[7], B) ? 0 : 2;
  }
  if (op == "lunopiv" && argc == 6) {
    if (!ReadMatrix(argv[4], A)) return 2;
    El::LU(A);
    return WriteMatrix(argv[5], A) ? 0 : 2;
  }
  if (op == "lufull" && argc == 8) {
    if (!ReadMatrix(argv[4], A)) return 2;
    El::Permutation Q;
    El::LU(A, P, Q);
    return (WriteMatrix(argv[5], A) && WritePivots(argv[6], P) && WritePivots(argv[7], Q))
               ? 0 : 2;
  }
  if (op == "lufullsolve" && argc == 11) {
    if (!ReadMatrix(argv[5], A) || !ReadMatrix(argv[6], B)) return 2;
    El::Permutation Q;
    El::LU(A, P, Q);
    El::lu::SolveAfter(Orient(argv[4]), A, P, Q, B);
    return (WriteMatrix(argv[7], A) && WritePivots(argv[8], P) && WritePivots(argv[9], Q) &&
            WriteMatrix(argv[10], B)) ? 0 : 2;
  }
  if (op == "inverse" && argc == 6) {
    if (!ReadMatrix(argv[4], A)) return 2;
    El::Inverse(A);
    return WriteMatrix(argv[5], A) ? 0 : 2;
  }
  if (op == "onecond" && argc == 6) {
    if (!ReadMatrix(argv[4], A)) return 2;
    El::Matrix<T> c(1, 1);
    c(0, 0) = El::OneCondition(A);
    return WriteMatrix(argv[5], c) ? 0 : 2;
  }
  if (op == "write" && argc == 7) {
    if (!ReadMatrix(argv[6], A)) return 2;
    El::Write(A, argv[5], argv[4][0] == 'd' ? El::BINARY_FLAT : El::BINARY);
    return 0;
  }
  if (op == "read" && argc == 6) {
    El::Read(A, argv[4]);
    return WriteMatrix(argv[5], A) ? 0 : 2;
  }
  if (op == "lutime" && argc == 6) {
    El::Matrix<T> A0;
    if (!ReadMatrix(argv[4], A0)) return 2;
    const int reps = std::atoi(argv[5]);
    double best = 1e300;
    for (int r = 0; r < reps; ++r) {
      A = A0;
      auto t0 = std::chrono::steady_clock::now();
      El::LU(A, P);
      auto t1 = std::chrono::steady_clock::now();
      best = std::min(best, std::chrono::duration<double>(t1 - t0).count());
    }
    std::printf("%.9f\n", best);
    return 0;
  }
  std::fprintf(stderr, "elref: bad arguments for op %s\n", op.c_str());
  return 2;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: elref <d|s> <op> <nb> ...\n");
    return 2;
  }
  try {
    if (argv[1][0] == 's') return Run<float>(argc, argv);
    return Run<double>(argc, argv);
  } catch (El::SingularMatrixException& e) {
    std::fprintf(stderr, "SingularMatrixException: %s\n", e.what());
    return 3;
  } catch (El::NonHPDMatrixException& e) {
    std::fprintf(stderr, "NonHPDMatrixException: %s\n", e.what());
    return 4;
  } catch (std::exception& e) {
    std::fprintf(stderr, "exception: %s\n", e.what());
    return 5;
  }
}
