/*
 * El_gb300.hpp — C++ drop-in for Elemental's sequential dense
 * factor-and-solve path, backed by the GB300 kernels of libelgb300.so.
 *
 * Same names, signatures, layouts and exceptions as the reference:
 *   El::Matrix<T>            include/El/core/Matrix/decl.hpp:17-241
 *   El::IR / ALL / View      include/El/core/types.hpp:15-68, View/decl.hpp:89-124
 *   El::Permutation          include/El/core/Permutation.hpp:14-126
 *   El::LU(A, P)             include/El/lapack_like/factor.hpp:376
 *   El::LU(A) (no pivoting)  include/El/lapack_like/factor.hpp:367
 *   El::LU(A, P, Q) (full)   include/El/lapack_like/factor.hpp:384-387
 *   El::Inverse(A)           include/El/lapack_like/funcs.hpp:68
 *   El::OneCondition(A)      include/El/lapack_like/props.hpp:37
 *   El::Read / El::Write     include/El/io.hpp:117,141 (BINARY, BINARY_FLAT)
 *   El::lu::SolveAfter       include/El/lapack_like/factor.hpp:434
 *   El::Cholesky(uplo, A)    include/El/lapack_like/factor.hpp:22
 *   El::cholesky::SolveAfter include/El/lapack_like/factor.hpp:63 (and :76-81 with P)
 *   El::Cholesky(uplo, A, P) include/El/lapack_like/factor.hpp:37
 *   El::LinearSolve(A, B)    include/El/lapack_like/solve.hpp:20
 *   El::HPDSolve             include/El/lapack_like/solve.hpp:190
 *   El::hpd_solve::Overwrite include/El/lapack_like/solve.hpp:213-228
 *   El::Blocksize / SetBlocksize / PushBlocksizeStack / PopBlocksizeStack
 *                            src/blas_like/blocksizes.cpp:37-60
 * Matrices live in host memory (as El::Matrix does); each call moves them to
 * the GPU, runs the device path and moves the results back.  Pinned host
 * buffers (Attach to cudaMallocHost memory) make those copies fast.
 */
#ifndef EL_GB300_HPP
#define EL_GB300_HPP

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace El {

typedef int Int;

enum UpperOrLower { LOWER, UPPER };
enum Orientation { NORMAL, TRANSPOSE, ADJOINT };
// Matrix file formats, in the reference's order (include/El/core/types.hpp,
// ElFileFormat include/El/core/types.h:237-251); BINARY and BINARY_FLAT are
// on this path.
enum FileFormat {
  AUTO, ASCII, ASCII_MATLAB, BINARY, BINARY_FLAT, BMP, JPG, JPEG, MATRIX_MARKET, PNG, PPM,
  XBM, XPM, FileFormat_MAX
};

// Index ranges [beg, end) (include/El/core/types.hpp:15-68): IR(i) is the one
// index i, END stands for the extent of the dimension it is applied to.
template <typename T>
struct Range {
  T beg, end;
  Range() : beg(0), end(0) {}
  Range(T begArg, T endArg) : beg(begArg), end(endArg) {}
};

static const Int END = -100;

template <>
struct Range<Int> {
  Int beg, end;
  Range() : beg(0), end(0) {}
  Range(Int index) : beg(index), end(index + 1) {}
  Range(Int begArg, Int endArg) : beg(begArg), end(endArg) {}
  Range<Int> operator+(Int shift) const {
    if (end == END) throw std::logic_error("Unsupported shift");
    return Range<Int>(beg + shift, end + shift);
  }
  Range<Int> operator-(Int shift) const {
    if (end == END) throw std::logic_error("Unsupported shift");
    return Range<Int>(beg - shift, end - shift);
  }
};
typedef Range<Int> IR;
static const IR ALL(0, END);

// Exception types of the reference (include/El/core/environment/decl.hpp:209-231).
class SingularMatrixException : public std::runtime_error {
 public:
  SingularMatrixException(const char* msg = "Matrix was singular")
      : std::runtime_error(msg) {}
};
class NonHPDMatrixException : public std::runtime_error {
 public:
  NonHPDMatrixException(const char* msg = "Matrix was not HPD")
      : std::runtime_error(msg) {}
};

template <typename T>
class Matrix {
 public:
  Matrix() {}
  Matrix(Int height, Int width) { Resize(height, width); }
  Matrix(Int height, Int width, Int ldim) { Resize(height, width, ldim); }
  Matrix(const Matrix<T>& A) { *this = A; }
  // A moved matrix keeps its kind: a view stays a view of the same buffer
  // (include/El/core/Matrix/impl.hpp:77-81).
  Matrix(Matrix<T>&& A) noexcept
      : height_(A.height_), width_(A.width_), ldim_(A.ldim_), buf_(A.buf_), cbuf_(A.cbuf_),
        viewing_(A.viewing_), locked_(A.locked_), mem_(std::move(A.mem_)) {
    A.Forget();
  }
  Matrix<T>& operator=(const Matrix<T>& A);
  // Moving into or out of a view copies the entries (impl.hpp:243-260).
  Matrix<T>& operator=(Matrix<T>&& A) {
    if (this == &A) return *this;
    if (viewing_ || A.viewing_) return *this = static_cast<const Matrix<T>&>(A);
    mem_.swap(A.mem_);
    height_ = A.height_;
    width_ = A.width_;
    ldim_ = A.ldim_;
    buf_ = A.buf_;
    cbuf_ = A.cbuf_;
    locked_ = false;
    A.Forget();
    A.mem_.clear();
    return *this;
  }

  // A view of rows I and columns J (decl.hpp:79-80); of a locked matrix, or
  // through a const matrix, a locked view.
  Matrix<T> operator()(Range<Int> I, Range<Int> J) {
    Matrix<T> V;
    Sub(I, J);
    if (locked_)
      V.LockedAttach(I.end - I.beg, J.end - J.beg, LockedBuffer(I.beg, J.beg), ldim_);
    else
      V.Attach(I.end - I.beg, J.end - J.beg, Buffer(I.beg, J.beg), ldim_);
    return V;
  }
  const Matrix<T> operator()(Range<Int> I, Range<Int> J) const {
    Matrix<T> V;
    Sub(I, J);
    V.LockedAttach(I.end - I.beg, J.end - J.beg, LockedBuffer(I.beg, J.beg), ldim_);
    return V;
  }

  void Empty();
  void Resize(Int height, Int width);
  void Resize(Int height, Int width, Int ldim);
  void Attach(Int height, Int width, T* buffer, Int ldim);
  void LockedAttach(Int height, Int width, const T* buffer, Int ldim);

  Int Height() const { return height_; }
  Int Width() const { return width_; }
  Int LDim() const { return ldim_; }
  bool Viewing() const { return viewing_; }
  bool Locked() const { return locked_; }

  T* Buffer();
  T* Buffer(Int i, Int j) { return Buffer() + i + (long)j * ldim_; }
  const T* LockedBuffer() const { return cbuf_; }
  const T* LockedBuffer(Int i, Int j) const { return cbuf_ + i + (long)j * ldim_; }

  T Get(Int i, Int j) const { return cbuf_[i + (long)j * ldim_]; }
  void Set(Int i, Int j, T alpha) { Buffer()[i + (long)j * ldim_] = alpha; }
  T& operator()(Int i, Int j) { return Buffer()[i + (long)j * ldim_]; }
  const T& operator()(Int i, Int j) const { return cbuf_[i + (long)j * ldim_]; }

  // Resolves END and checks that rows I, columns J lie inside the matrix.
  void Sub(Range<Int>& I, Range<Int>& J) const {
    if (I.end == END) I.end = height_;
    if (J.end == END) J.end = width_;
    if (I.beg < 0 || J.beg < 0 || I.end < I.beg || J.end < J.beg || I.end > height_ ||
        J.end > width_)
      throw std::logic_error("Trying to view outside of a Matrix");
  }

 private:
  void Reallocate(Int ldim);
  void Forget() {
    height_ = width_ = 0;
    ldim_ = 1;
    buf_ = nullptr;
    cbuf_ = nullptr;
    viewing_ = locked_ = false;
  }

  Int height_ = 0, width_ = 0, ldim_ = 1;
  T* buf_ = nullptr;
  const T* cbuf_ = nullptr;
  bool viewing_ = false, locked_ = false;
  std::vector<T> mem_;
};

// Views of a contiguous submatrix (include/El/core/View/decl.hpp:89-124,
// impl.hpp:274-387): A becomes a view of B's rows I and columns J.
template <typename T>
void View(Matrix<T>& A, Matrix<T>& B, Range<Int> I, Range<Int> J) {
  B.Sub(I, J);
  if (B.Locked())
    A.LockedAttach(I.end - I.beg, J.end - J.beg, B.LockedBuffer(I.beg, J.beg), B.LDim());
  else
    A.Attach(I.end - I.beg, J.end - J.beg, B.Buffer(I.beg, J.beg), B.LDim());
}
template <typename T>
void LockedView(Matrix<T>& A, const Matrix<T>& B, Range<Int> I, Range<Int> J) {
  B.Sub(I, J);
  A.LockedAttach(I.end - I.beg, J.end - J.beg, B.LockedBuffer(I.beg, J.beg), B.LDim());
}
template <typename T>
void View(Matrix<T>& A, Matrix<T>& B, Int i, Int j, Int height, Int width) {
  View(A, B, IR(i, i + height), IR(j, j + width));
}
template <typename T>
void LockedView(Matrix<T>& A, const Matrix<T>& B, Int i, Int j, Int height, Int width) {
  LockedView(A, B, IR(i, i + height), IR(j, j + width));
}
template <typename T>
Matrix<T> View(Matrix<T>& B, Range<Int> I, Range<Int> J) {
  Matrix<T> A;
  View(A, B, I, J);
  return A;
}
template <typename T>
Matrix<T> LockedView(const Matrix<T>& B, Range<Int> I, Range<Int> J) {
  Matrix<T> A;
  LockedView(A, B, I, J);
  return A;
}

class Permutation {
 public:
  void Empty();
  void MakeIdentity(Int size);
  void ReserveSwaps(Int maxSwaps);
  // Appends the swap (origin, dest).  While every origin equals the number of
  // swaps before it the origins stay implicit (0, 1, 2, ...); the first other
  // origin makes them explicit (src/lapack_like/perm/Permutation.cpp:205-250).
  void Swap(Int origin, Int dest);
  void SwapSequence(const Permutation& P, Int offset = 0);
  void SwapSequence(const Matrix<Int>& swapOrigins, const Matrix<Int>& swapDests,
                    Int offset = 0);
  void ImplicitSwapSequence(const Matrix<Int>& swapDests, Int offset = 0);

  Int Height() const { return size_; }
  Int Width() const { return size_; }
  bool Parity() const;
  bool IsSwapSequence() const { return true; }
  bool IsImplicitSwapSequence() const { return implicit_; }

  // The origins of the recorded swaps (0, 1, ... when implicit).
  const Matrix<Int> SwapOrigins() const;
  const Matrix<Int> SwapDestinations() const;
  template <typename T>
  void PermuteRows(Matrix<T>& A, Int offset = 0) const;
  template <typename T>
  void InversePermuteRows(Matrix<T>& A, Int offset = 0) const;
  void ExplicitVector(Matrix<Int>& p) const;

  // Number of swaps recorded and direct access to their destinations (whose
  // origins are 0, 1, ... only when IsImplicitSwapSequence()).
  Int NumSwaps() const { return numSwaps_; }
  const Int* SwapDestBuffer() const { return dests_.data(); }
  // Replaces the swap sequence by `numSwaps` destinations (origins 0..).
  void SetSwapSequence(Int size, const Int* dests, Int numSwaps);
  // The destinations of an implicit-origin sequence of n swaps that permutes
  // n rows exactly as this one does (n >= Height()).
  std::vector<Int> ImplicitSwapDests(Int n) const;

 private:
  Int Origin(Int k) const { return implicit_ ? k : origins_[k]; }

  Int size_ = 0;
  Int numSwaps_ = 0;
  bool implicit_ = true;
  std::vector<Int> dests_;
  std::vector<Int> origins_;  // used once the origins are explicit
};

Int Blocksize();
void SetBlocksize(Int blocksize);
void PushBlocksizeStack(Int blocksize);
void PopBlocksizeStack();

template <typename F>
void LU(Matrix<F>& A, Permutation& P);

// LU with full pivoting (P rows, Q columns); SingularMatrixException at an
// exact zero pivot (the swaps of that step are recorded).
template <typename F>
void LU(Matrix<F>& A, Permutation& P, Permutation& Q);

// LU without pivoting; throws SingularMatrixException at an exact zero pivot.
template <typename F>
void LU(Matrix<F>& A);

// A := inv(A) (LU with partial pivoting); SingularMatrixException at an exact
// zero pivot, LogicError for a non-square A.
template <typename F>
void Inverse(Matrix<F>& A);

// ||A||_1 ||inv(A)||_1; +infinity for a singular A.
template <typename F>
F OneCondition(const Matrix<F>& A);

// Matrix files.  BINARY (basename.bin): Int height, Int width, then the
// entries column by column; BINARY_FLAT (basename.dat): the entries only,
// read into A's current shape.  AUTO picks the format from the extension.
// Other formats throw std::logic_error; I/O failures std::runtime_error.
template <typename T>
void Read(Matrix<T>& A, const std::string& filename, FileFormat format = AUTO);
template <typename T>
void Write(const Matrix<T>& A, const std::string& basename = "matrix",
           FileFormat format = BINARY, const std::string& title = "");

namespace lu {
template <typename F>
void SolveAfter(Orientation orientation, const Matrix<F>& A, const Permutation& P,
                Matrix<F>& B);
template <typename F>
void SolveAfter(Orientation orientation, const Matrix<F>& A, const Permutation& P,
                const Permutation& Q, Matrix<F>& B);
}  // namespace lu

template <typename F>
void Cholesky(UpperOrLower uplo, Matrix<F>& A);

// Cholesky with diagonal pivoting, P A P^T = L L^T (or U^T U).
template <typename F>
void Cholesky(UpperOrLower uplo, Matrix<F>& A, Permutation& P);

namespace cholesky {
template <typename F>
void SolveAfter(UpperOrLower uplo, Orientation orientation, const Matrix<F>& A,
                Matrix<F>& B);
template <typename F>
void SolveAfter(UpperOrLower uplo, Orientation orientation, const Matrix<F>& A,
                const Permutation& P, Matrix<F>& B);
}  // namespace cholesky

template <typename F>
void LinearSolve(const Matrix<F>& A, Matrix<F>& B);

template <typename F>
void HPDSolve(UpperOrLower uplo, Orientation orientation, const Matrix<F>& A, Matrix<F>& B);

namespace hpd_solve {
// HPDSolve without the copy of A: A is overwritten by its Cholesky factor
// (include/El/lapack_like/solve.hpp:213-228, src/lapack_like/solve/HPD.cpp:15-25).
template <typename F>
void Overwrite(UpperOrLower uplo, Orientation orientation, Matrix<F>& A, Matrix<F>& B) {
  Cholesky(uplo, A);
  cholesky::SolveAfter(uplo, orientation, A, B);
}
}  // namespace hpd_solve

}  // namespace El

#include "elgb300.h"

namespace El {

// Added form (no counterpart in the reference): LinearSolve through the
// mixed-precision path (tensor-core low-precision LU + LU-IR / GMRES-IR with
// an FP64 residual, FP64 LU fallback).  ctrl may be null.
void LinearSolveMixed(const Matrix<double>& A, Matrix<double>& B,
                      const ElGBRefineCtrl* ctrl = nullptr, ElGBRefineInfo* info = nullptr);

// Added (no counterpart in the reference): the host-side phases of the last
// completed host-matrix call in milliseconds: t[0] uploads, t[1] the device
// work with its synchronisation, t[2] downloads.
void LastHostCallTimes(double* t);

}  // namespace El

#endif  // EL_GB300_HPP
