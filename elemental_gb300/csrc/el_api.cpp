// El-compatible host layer (include/El_gb300.hpp) and the Elemental C ABI
// subset (include/El_gb300.h).  Host matrices are staged into device memory,
// the device path of include/elgb300.h runs, results come back; the numerical
// failures become the reference's exceptions, and the C entry points map
// exceptions to ElError exactly as the reference's EL_TRY does
// (include/El/core/CReflect.hpp:12-26).
#include <cuda_runtime.h>
#include <sys/mman.h>

#include <algorithm>
#include <chrono>
#include <fstream>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/El_gb300.h"
#include "../../include/El_gb300.hpp"
#include "../../include/elgb300.h"

namespace El {

// ---------------------------------------------------------------------------
// Matrix<T>
// ---------------------------------------------------------------------------
template <typename T>
Matrix<T>& Matrix<T>::operator=(const Matrix<T>& A) {
  if (this == &A) return *this;
  // a locked matrix has no writable buffer: the reference's Copy reaches it
  // through Buffer(), which raises the same LogicError
  if (locked_) throw std::logic_error("Cannot return non-const buffer of locked Matrix");
  Resize(A.Height(), A.Width());
  T* dst = Buffer();
  for (Int j = 0; j < width_; ++j)
    for (Int i = 0; i < height_; ++i) dst[i + (long)j * ldim_] = A.Get(i, j);
  return *this;
}

template <typename T>
void Matrix<T>::Empty() {
  height_ = width_ = 0;
  ldim_ = 1;
  buf_ = nullptr;
  cbuf_ = nullptr;
  viewing_ = locked_ = false;
  mem_.clear();
  mem_.shrink_to_fit();
}

// The reference's Resize_ (include/El/core/Matrix/impl.hpp:698-716): the
// leading dimension and the entries stay unless the new shape needs more
// rows than the leading dimension or more columns than before; a view may
// only shrink (impl.hpp:101-115).
template <typename T>
void Matrix<T>::Resize(Int height, Int width) {
  if (height < 0 || width < 0) throw std::logic_error("Matrix::Resize: invalid dimensions");
  if (viewing_ && (height > height_ || width > width_))
    throw std::logic_error("Cannot increase the size of a view");
  const bool realloc = !viewing_ && (height > ldim_ || width > width_);
  height_ = height;
  width_ = width;
  if (realloc) Reallocate(std::max(height, 1));
}

template <typename T>
void Matrix<T>::Resize(Int height, Int width, Int ldim) {
  if (height < 0 || width < 0 || ldim < std::max(height, 1))
    throw std::logic_error("Matrix::Resize: invalid dimensions");
  if (viewing_ && (height > height_ || width > width_ || ldim != ldim_))
    throw std::logic_error("Cannot increase the size of a view");
  const bool realloc = !viewing_ && (height > ldim_ || width > width_ || ldim != ldim_);
  height_ = height;
  width_ = width;
  if (realloc) Reallocate(ldim);
}

// Storage for ldim x width entries: as the reference's Memory::Require
// (include/El/core/Memory/impl.hpp:69-100), a buffer that is already large
// enough is kept as it is; a larger one replaces it (zero-filled here) and
// the old entries are not carried over.
template <typename T>
void Matrix<T>::Reallocate(Int ldim) {
  ldim_ = ldim;
  const size_t need = (size_t)ldim * std::max(width_, 0);
  if (need > mem_.size()) mem_.assign(need, T(0));
  buf_ = mem_.data();
  cbuf_ = buf_;
}

template <typename T>
void Matrix<T>::Attach(Int height, Int width, T* buffer, Int ldim) {
  if (height < 0 || width < 0 || ldim < std::max(height, 1))
    throw std::logic_error("Matrix::Attach: invalid dimensions");
  mem_.clear();
  height_ = height;
  width_ = width;
  ldim_ = ldim;
  buf_ = buffer;
  cbuf_ = buffer;
  viewing_ = true;
  locked_ = false;
}

template <typename T>
void Matrix<T>::LockedAttach(Int height, Int width, const T* buffer, Int ldim) {
  if (height < 0 || width < 0 || ldim < std::max(height, 1))
    throw std::logic_error("Matrix::LockedAttach: invalid dimensions");
  mem_.clear();
  height_ = height;
  width_ = width;
  ldim_ = ldim;
  buf_ = nullptr;
  cbuf_ = buffer;
  viewing_ = true;
  locked_ = true;
}

template <typename T>
T* Matrix<T>::Buffer() {
  if (locked_) throw std::logic_error("Cannot return non-const buffer of locked Matrix");
  return buf_;
}

template class Matrix<Int>;
template class Matrix<float>;
template class Matrix<double>;

// ---------------------------------------------------------------------------
// Permutation: a swap sequence, origins implicit (0, 1, 2, ...) until a swap
// names another origin (src/lapack_like/perm/Permutation.cpp:166-303,
// 436-450, 544-631, 731-745).  It never becomes an arbitrary permutation:
// past the reserved count the sequence grows.
// ---------------------------------------------------------------------------
void Permutation::Empty() {
  size_ = 0;
  numSwaps_ = 0;
  implicit_ = true;
  dests_.clear();
  origins_.clear();
}

void Permutation::MakeIdentity(Int size) {
  size_ = size;
  numSwaps_ = 0;
  implicit_ = true;
  origins_.clear();
}

void Permutation::ReserveSwaps(Int maxSwaps) {
  if ((Int)dests_.size() < maxSwaps) dests_.resize(maxSwaps);
}

void Permutation::Swap(Int origin, Int dest) {
  if (origin < 0 || origin >= size_ || dest < 0 || dest >= size_)
    throw std::logic_error("Permutation::Swap: index out of range");
  if ((Int)dests_.size() <= numSwaps_) dests_.resize(numSwaps_ + 1);
  if (implicit_ && origin != numSwaps_) {
    implicit_ = false;
    origins_.resize(numSwaps_);
    for (Int k = 0; k < numSwaps_; ++k) origins_[k] = k;
  }
  if (!implicit_) {
    if ((Int)origins_.size() <= numSwaps_) origins_.resize(numSwaps_ + 1);
    origins_[numSwaps_] = origin;
  }
  dests_[numSwaps_++] = dest;
}

void Permutation::SwapSequence(const Permutation& P, Int offset) {
  const Int count = P.numSwaps_;  // P may be *this
  for (Int k = 0; k < count; ++k) Swap(P.Origin(k) + offset, P.dests_[k] + offset);
}

void Permutation::SwapSequence(const Matrix<Int>& swapOrigins, const Matrix<Int>& swapDests,
                               Int offset) {
  if (swapOrigins.Height() != swapDests.Height())
    throw std::logic_error("Permutation::SwapSequence: origins and destinations differ in size");
  for (Int k = 0; k < swapDests.Height(); ++k)
    Swap(swapOrigins.Get(k, 0) + offset, swapDests.Get(k, 0) + offset);
}

void Permutation::ImplicitSwapSequence(const Matrix<Int>& swapDests, Int offset) {
  const Int before = numSwaps_;
  for (Int k = 0; k < swapDests.Height(); ++k) Swap(before + k, swapDests.Get(k, 0) + offset);
}

bool Permutation::Parity() const {
  bool p = false;
  for (Int j = 0; j < numSwaps_; ++j)
    if (dests_[j] != Origin(j)) p = !p;
  return p;
}

const Matrix<Int> Permutation::SwapOrigins() const {
  Matrix<Int> o(numSwaps_, 1);
  for (Int j = 0; j < numSwaps_; ++j) o(j, 0) = Origin(j);
  return o;
}

const Matrix<Int> Permutation::SwapDestinations() const {
  Matrix<Int> d(numSwaps_, 1);
  for (Int j = 0; j < numSwaps_; ++j) d(j, 0) = dests_[j];
  return d;
}

template <typename T>
static void RowSwapHost(Matrix<T>& A, Int to, Int from) {
  if (to == from) return;
  T* b = A.Buffer();
  const Int ld = A.LDim();
  for (Int j = 0; j < A.Width(); ++j) std::swap(b[to + (long)j * ld], b[from + (long)j * ld]);
}

template <typename T>
void Permutation::PermuteRows(Matrix<T>& A, Int offset) const {
  if (A.Height() == 0 || A.Width() == 0) return;
  for (Int j = 0; j < numSwaps_; ++j) RowSwapHost(A, Origin(j) + offset, dests_[j] + offset);
}

template <typename T>
void Permutation::InversePermuteRows(Matrix<T>& A, Int offset) const {
  if (A.Height() == 0 || A.Width() == 0) return;
  for (Int j = numSwaps_ - 1; j >= 0; --j)
    RowSwapHost(A, Origin(j) + offset, dests_[j] + offset);
}

void Permutation::ExplicitVector(Matrix<Int>& p) const {
  p.Resize(size_, 1);
  for (Int i = 0; i < size_; ++i) p(i, 0) = i;
  PermuteRows(p);
}

std::vector<Int> Permutation::ImplicitSwapDests(Int n) const {
  if (size_ > n) throw std::logic_error("Permutation is larger than the row count");
  std::vector<Int> d(n);
  if (implicit_) {
    for (Int i = 0; i < n; ++i) d[i] = i < numSwaps_ ? dests_[i] : i;
    return d;
  }
  // row k of P A is row p[k] of A: swap row k with the row now holding p[k]
  Matrix<Int> p;
  ExplicitVector(p);
  std::vector<Int> lab(n), pos(n);
  for (Int i = 0; i < n; ++i) lab[i] = pos[i] = i;
  for (Int k = 0; k < n; ++k) {
    const Int j = pos[k < size_ ? p.Get(k, 0) : k];
    d[k] = j;
    std::swap(lab[k], lab[j]);
    pos[lab[k]] = k;
    pos[lab[j]] = j;
  }
  return d;
}

void Permutation::SetSwapSequence(Int size, const Int* dests, Int numSwaps) {
  size_ = size;
  numSwaps_ = numSwaps;
  implicit_ = true;
  origins_.clear();
  dests_.assign(dests, dests + numSwaps);
}

template void Permutation::PermuteRows<Int>(Matrix<Int>&, Int) const;
template void Permutation::PermuteRows<float>(Matrix<float>&, Int) const;
template void Permutation::PermuteRows<double>(Matrix<double>&, Int) const;
template void Permutation::InversePermuteRows<Int>(Matrix<Int>&, Int) const;
template void Permutation::InversePermuteRows<float>(Matrix<float>&, Int) const;
template void Permutation::InversePermuteRows<double>(Matrix<double>&, Int) const;

// ---------------------------------------------------------------------------
// Blocksize stack (src/blas_like/blocksizes.cpp:37-60)
// ---------------------------------------------------------------------------
namespace {
std::vector<Int>& BlocksizeStack() {
  static std::vector<Int> s{128};
  return s;
}
}  // namespace

Int Blocksize() { return BlocksizeStack().back(); }
void SetBlocksize(Int blocksize) {
  BlocksizeStack().back() = blocksize;
  ElGBSetBlocksize(blocksize);
}
void PushBlocksizeStack(Int blocksize) {
  BlocksizeStack().push_back(blocksize);
  ElGBSetBlocksize(blocksize);
}
void PopBlocksizeStack() {
  if (BlocksizeStack().size() > 1) BlocksizeStack().pop_back();
  ElGBSetBlocksize(BlocksizeStack().back());
}

// ---------------------------------------------------------------------------
// Device staging shared by the host-matrix entry points
// ---------------------------------------------------------------------------
namespace {

using Clock = std::chrono::steady_clock;

struct Staging {
  std::mutex mu;
  ElGBContext ctx = nullptr;
  int device = -1;
  void* buf = nullptr;
  size_t bytes = 0;
  cudaStream_t copy[2] = {nullptr, nullptr};  // host <-> device copy streams
  // host-side phases of the current / last call (ElGBLastHostCallTimes)
  double up_ms = 0, down_ms = 0;
  double last[3] = {0, 0, 0};
};

Staging& St() {
  static Staging s;
  return s;
}

void Check(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

double MsSince(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// Serialises the host-matrix entry points (they share the staging buffer)
// and records the call's host-side phases: upload, download, and the rest
// (the device work and its synchronisation).
struct CallGuard {
  std::lock_guard<std::mutex> lk;
  Clock::time_point t0;
  CallGuard() : lk(St().mu), t0(Clock::now()) { St().up_ms = St().down_ms = 0; }
  ~CallGuard() {
    Staging& s = St();
    const double tot = MsSince(t0);
    s.last[0] = s.up_ms;
    s.last[1] = std::max(tot - s.up_ms - s.down_ms, 0.0);
    s.last[2] = s.down_ms;
  }
};

ElGBContext Ctx() {
  Staging& s = St();
  int dev = 0;
  Check(cudaGetDevice(&dev), "cudaGetDevice");
  if (s.ctx && s.device != dev) {
    ElGBDestroy(s.ctx);
    s.ctx = nullptr;
    if (s.buf) cudaFree(s.buf);
    s.buf = nullptr;
    s.bytes = 0;
    for (auto& c : s.copy) {
      if (c) cudaStreamDestroy(c);
      c = nullptr;
    }
  }
  if (!s.ctx) {
    if (ElGBCreate(&s.ctx, dev) != 0) throw std::runtime_error("no usable CUDA device");
    s.device = dev;
    for (auto& c : s.copy) Check(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking), "stream");
  }
  return s.ctx;
}

char* Dev(size_t bytes) {
  Staging& s = St();
  if (bytes > s.bytes) {
    if (s.buf) cudaFree(s.buf);
    s.buf = nullptr;
    s.bytes = 0;
    Check(cudaMalloc(&s.buf, bytes), "cudaMalloc");
    s.bytes = bytes;
  }
  return static_cast<char*>(s.buf);
}

size_t Al(size_t b) { return (b + 255) & ~size_t(255); }

// The swap destinations (origins implicit 0, 1, ..., n - 1) that replay P
// on n rows, as the device's swap kernels take them; every destination is
// checked to lie in [0, n) before it can reach the device.
std::vector<int> DevicePivots(const Permutation& P, Int n) {
  const std::vector<Int> d = P.ImplicitSwapDests(n);
  for (Int i = 0; i < n; ++i)
    if (d[i] < 0 || d[i] >= n) throw std::logic_error("Permutation swap out of range");
  return std::vector<int>(d.begin(), d.end());
}

// Host -> device copy of a column-major matrix: blocks of columns of about
// 64 MiB, alternating between two copy streams so that both copy engines of
// the direction can run, one call per block (a contiguous matrix takes plain
// 1-D copies), then a wait for both streams.  The legacy default stream is
// drained as well: a synchronous copy from pageable memory (the small pivot
// copies some callers issue just before) may return once its data is staged,
// before its DMA ends, and the factor-and-solve work runs on the context's
// non-blocking stream, which is not ordered after the legacy stream.
template <typename T>
void Upload(ElGBContext, T* d, const Matrix<T>& A) {
  if (A.Height() == 0 || A.Width() == 0) return;
  Staging& s = St();
  const Clock::time_point t0 = Clock::now();
  const Int h = A.Height(), w = A.Width(), ld = A.LDim();
  const size_t colb = sizeof(T) * (size_t)h;
  const Int cols = std::max<Int>(1, (Int)(((size_t)64 << 20) / colb));
  int k = 0;
  for (Int j = 0; j < w; j += cols, ++k) {
    const Int nc = std::min(cols, w - j);
    cudaStream_t st = s.copy[k & 1];
    if (ld == h || nc == 1)
      Check(cudaMemcpyAsync(d + (size_t)j * h, A.LockedBuffer(0, j), colb * nc,
                            cudaMemcpyHostToDevice, st), "upload");
    else
      Check(cudaMemcpy2DAsync(d + (size_t)j * h, colb, A.LockedBuffer(0, j), sizeof(T) * ld,
                              colb, nc, cudaMemcpyHostToDevice, st), "upload");
  }
  for (cudaStream_t st : s.copy) Check(cudaStreamSynchronize(st), "upload");
  Check(cudaStreamSynchronize(cudaStreamLegacy), "upload");
  s.up_ms += MsSince(t0);
}

template <typename T>
void Download(Matrix<T>& A, const T* d) {
  if (A.Height() == 0 || A.Width() == 0) return;
  const Clock::time_point t0 = Clock::now();
  Check(cudaMemcpy2D(A.Buffer(), sizeof(T) * A.LDim(), d, sizeof(T) * A.Height(),
                     sizeof(T) * A.Height(), A.Width(), cudaMemcpyDeviceToHost),
        "download");
  St().down_ms += MsSince(t0);
}

void CheckStatus(ElGBContext ctx, bool cholesky) {
  int info = 0, err = 0;
  if (ElGBStatus(ctx, &info, &err) != 0) throw std::runtime_error("CUDA failure");
  if (err) throw std::runtime_error("device-side wait timed out");
  if (info) {
    if (cholesky) throw NonHPDMatrixException("A was not numerically HPD");
    throw SingularMatrixException();
  }
}

void CheckRc(int rc) {
  if (rc == 3) throw std::invalid_argument("invalid argument");
  if (rc != 0) throw std::runtime_error("GB300 factor-and-solve call failed");
}

template <typename F>
struct Dispatch;
template <>
struct Dispatch<double> {
  static int lu(ElGBContext c, int m, int n, double* A, int lda, int* p, int nb) {
    return ElGBLUPartialPiv_d(c, m, n, A, lda, p, nb);
  }
  static int lus(ElGBContext c, int o, int n, const double* A, int lda, const int* p, int q,
                 double* B, int ldb) {
    return ElGBSolveAfterLUPartialPiv_d(c, o, n, A, lda, p, q, B, ldb);
  }
  static int chol(ElGBContext c, int u, int n, double* A, int lda, int nb) {
    return ElGBCholesky_d(c, u, n, A, lda, nb);
  }
  static int chols(ElGBContext c, int u, int n, const double* A, int lda, int q, double* B,
                   int ldb) {
    return ElGBSolveAfterCholesky_d(c, u, n, A, lda, q, B, ldb);
  }
  static int lin(ElGBContext c, int n, const double* A, int lda, int q, double* B, int ldb,
                 int nb) {
    return ElGBLinearSolve_d(c, n, A, lda, q, B, ldb, nb);
  }
  static int hpd(ElGBContext c, int u, int n, const double* A, int lda, int q, double* B,
                 int ldb, int nb) {
    return ElGBHPDSolve_d(c, u, n, A, lda, q, B, ldb, nb);
  }
  static int lunopiv(ElGBContext c, int m, int n, double* A, int lda, int nb) {
    return ElGBLUNoPiv_d(c, m, n, A, lda, nb);
  }
  static int inv(ElGBContext c, int n, double* A, int lda, int nb) {
    return ElGBInverse_d(c, n, A, lda, nb);
  }
  static int cond1(ElGBContext c, int n, const double* A, int lda, int nb, double* k) {
    return ElGBOneCondition_d(c, n, A, lda, nb, k);
  }
  static int lufull(ElGBContext c, int m, int n, double* A, int lda, int* p, int* q) {
    return ElGBLUFullPiv_d(c, m, n, A, lda, p, q);
  }
  static int cholpiv(ElGBContext c, int u, int n, double* A, int lda, int* p) {
    return ElGBCholeskyPiv_d(c, u, n, A, lda, p);
  }
  static int cholpivs(ElGBContext c, int u, int n, const double* A, int lda, const int* p,
                      int nr, double* B, int ldb) {
    return ElGBSolveAfterCholeskyPiv_d(c, u, n, A, lda, p, nr, B, ldb);
  }
  static int lufulls(ElGBContext c, int o, int n, const double* A, int lda, const int* p,
                     const int* q, int nr, double* B, int ldb) {
    return ElGBSolveAfterLUFullPiv_d(c, o, n, A, lda, p, q, nr, B, ldb);
  }
};
template <>
struct Dispatch<float> {
  static int lu(ElGBContext c, int m, int n, float* A, int lda, int* p, int nb) {
    return ElGBLUPartialPiv_s(c, m, n, A, lda, p, nb);
  }
  static int lus(ElGBContext c, int o, int n, const float* A, int lda, const int* p, int q,
                 float* B, int ldb) {
    return ElGBSolveAfterLUPartialPiv_s(c, o, n, A, lda, p, q, B, ldb);
  }
  static int chol(ElGBContext c, int u, int n, float* A, int lda, int nb) {
    return ElGBCholesky_s(c, u, n, A, lda, nb);
  }
  static int chols(ElGBContext c, int u, int n, const float* A, int lda, int q, float* B,
                   int ldb) {
    return ElGBSolveAfterCholesky_s(c, u, n, A, lda, q, B, ldb);
  }
  static int lin(ElGBContext c, int n, const float* A, int lda, int q, float* B, int ldb,
                 int nb) {
    return ElGBLinearSolve_s(c, n, A, lda, q, B, ldb, nb);
  }
  static int hpd(ElGBContext c, int u, int n, const float* A, int lda, int q, float* B,
                 int ldb, int nb) {
    return ElGBHPDSolve_s(c, u, n, A, lda, q, B, ldb, nb);
  }
  static int lunopiv(ElGBContext c, int m, int n, float* A, int lda, int nb) {
    return ElGBLUNoPiv_s(c, m, n, A, lda, nb);
  }
  static int inv(ElGBContext c, int n, float* A, int lda, int nb) {
    return ElGBInverse_s(c, n, A, lda, nb);
  }
  static int cond1(ElGBContext c, int n, const float* A, int lda, int nb, double* k) {
    return ElGBOneCondition_s(c, n, A, lda, nb, k);
  }
  static int lufull(ElGBContext c, int m, int n, float* A, int lda, int* p, int* q) {
    return ElGBLUFullPiv_s(c, m, n, A, lda, p, q);
  }
  static int cholpiv(ElGBContext c, int u, int n, float* A, int lda, int* p) {
    return ElGBCholeskyPiv_s(c, u, n, A, lda, p);
  }
  static int cholpivs(ElGBContext c, int u, int n, const float* A, int lda, const int* p,
                      int nr, float* B, int ldb) {
    return ElGBSolveAfterCholeskyPiv_s(c, u, n, A, lda, p, nr, B, ldb);
  }
  static int lufulls(ElGBContext c, int o, int n, const float* A, int lda, const int* p,
                     const int* q, int nr, float* B, int ldb) {
    return ElGBSolveAfterLUFullPiv_s(c, o, n, A, lda, p, q, nr, B, ldb);
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// The path: El::LU, lu::SolveAfter, El::Cholesky, cholesky::SolveAfter,
// El::LinearSolve, El::HPDSolve
// ---------------------------------------------------------------------------
template <typename F>
void LU(Matrix<F>& A, Permutation& P) {
  CallGuard guard;
  const Int m = A.Height(), n = A.Width(), minDim = std::min(m, n);
  P.MakeIdentity(m);
  P.ReserveSwaps(minDim);
  if (minDim == 0) {
    P.SetSwapSequence(m, nullptr, 0);
    return;
  }
  ElGBContext ctx = Ctx();
  char* base = Dev(Al(sizeof(F) * (size_t)m * n) + Al(sizeof(int) * minDim));
  F* dA = reinterpret_cast<F*>(base);
  int* dP = reinterpret_cast<int*>(base + Al(sizeof(F) * (size_t)m * n));
  Upload(ctx, dA, A);
  CheckRc(Dispatch<F>::lu(ctx, m, n, dA, m, dP, Blocksize()));
  int info = 0, err = 0;
  if (ElGBStatus(ctx, &info, &err) != 0) throw std::runtime_error("CUDA failure");
  Download(A, dA);
  std::vector<Int> piv(minDim);
  Check(cudaMemcpy(piv.data(), dP, sizeof(int) * minDim, cudaMemcpyDeviceToHost), "pivots");
  if (err) throw std::runtime_error("device-side wait timed out");
  if (info) {
    // The reference stops at the failing column (LU/Panel.hpp:51-52) with
    // the swaps recorded up to and including it.
    P.SetSwapSequence(m, piv.data(), std::min<Int>(info, minDim));
    throw SingularMatrixException();
  }
  P.SetSwapSequence(m, piv.data(), minDim);
}

// El::LU(A, P, Q) with full pivoting (src/lapack_like/factor/LU.cpp:145-152).
template <typename F>
void LU(Matrix<F>& A, Permutation& P, Permutation& Q) {
  CallGuard guard;
  const Int m = A.Height(), n = A.Width(), minDim = std::min(m, n);
  P.MakeIdentity(m);
  Q.MakeIdentity(n);
  P.ReserveSwaps(minDim);
  Q.ReserveSwaps(minDim);
  if (minDim == 0) {
    P.SetSwapSequence(m, nullptr, 0);
    Q.SetSwapSequence(n, nullptr, 0);
    return;
  }
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)m * n), sp = Al(sizeof(int) * minDim);
  char* base = Dev(sa + 2 * sp);
  F* dA = reinterpret_cast<F*>(base);
  int* dP = reinterpret_cast<int*>(base + sa);
  int* dQ = reinterpret_cast<int*>(base + sa + sp);
  Upload(ctx, dA, A);
  CheckRc(Dispatch<F>::lufull(ctx, m, n, dA, m, dP, dQ));
  int info = 0, err = 0;
  if (ElGBStatus(ctx, &info, &err) != 0) throw std::runtime_error("CUDA failure");
  Download(A, dA);
  std::vector<Int> p(minDim), q(minDim);
  Check(cudaMemcpy(p.data(), dP, sizeof(int) * minDim, cudaMemcpyDeviceToHost), "pivots");
  Check(cudaMemcpy(q.data(), dQ, sizeof(int) * minDim, cudaMemcpyDeviceToHost), "pivots");
  if (err) throw std::runtime_error("device-side wait timed out");
  // the reference records step k's swaps before it finds the zero pivot
  const Int ns = info ? std::min<Int>(info, minDim) : minDim;
  P.SetSwapSequence(m, p.data(), ns);
  Q.SetSwapSequence(n, q.data(), ns);
  if (info) throw SingularMatrixException();
}

// El::LU(A) without pivoting (src/lapack_like/factor/LU.cpp:21-44).
template <typename F>
void LU(Matrix<F>& A) {
  CallGuard guard;
  const Int m = A.Height(), n = A.Width();
  if (std::min(m, n) == 0) return;
  ElGBContext ctx = Ctx();
  F* dA = reinterpret_cast<F*>(Dev(Al(sizeof(F) * (size_t)m * n)));
  Upload(ctx, dA, A);
  CheckRc(Dispatch<F>::lunopiv(ctx, m, n, dA, m, Blocksize()));
  CheckStatus(ctx, false);  // lu::Unb throws at an exact zero pivot (LU/Local.hpp:50-51)
  Download(A, dA);
}

// El::Inverse (src/lapack_like/funcs/Inverse/General.cpp:15-20).
template <typename F>
void Inverse(Matrix<F>& A) {
  if (A.Height() != A.Width()) throw std::logic_error("Cannot invert non-square matrices");
  CallGuard guard;
  const Int n = A.Height();
  if (n == 0) return;
  ElGBContext ctx = Ctx();
  F* dA = reinterpret_cast<F*>(Dev(Al(sizeof(F) * (size_t)n * n)));
  Upload(ctx, dA, A);
  CheckRc(Dispatch<F>::inv(ctx, n, dA, n, Blocksize()));
  CheckStatus(ctx, false);
  Download(A, dA);
}

// El::OneCondition (src/lapack_like/props/Condition/One.cpp:12-24).
template <typename F>
F OneCondition(const Matrix<F>& A) {
  if (A.Height() != A.Width()) throw std::logic_error("OneCondition needs a square matrix");
  CallGuard guard;
  const Int n = A.Height();
  if (n == 0) return F(0);
  ElGBContext ctx = Ctx();
  F* dA = reinterpret_cast<F*>(Dev(Al(sizeof(F) * (size_t)n * n)));
  Upload(ctx, dA, A);
  double k = 0.0;
  CheckRc(Dispatch<F>::cond1(ctx, n, dA, n, Blocksize(), &k));
  return static_cast<F>(k);
}

namespace lu {
template <typename F>
void SolveAfter(Orientation orientation, const Matrix<F>& A, const Permutation& P,
                Matrix<F>& B) {
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  if (A.Height() != B.Height()) throw std::logic_error("A and B must be the same height");
  CallGuard guard;
  const Int n = A.Height(), q = B.Width();
  if (n == 0 || q == 0) return;
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)n * n), sb = Al(sizeof(F) * (size_t)n * q);
  char* base = Dev(sa + sb + Al(sizeof(int) * n));
  F* dA = reinterpret_cast<F*>(base);
  F* dB = reinterpret_cast<F*>(base + sa);
  int* dP = reinterpret_cast<int*>(base + sa + sb);
  const std::vector<int> piv = DevicePivots(P, n);
  Check(cudaMemcpy(dP, piv.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "pivots");
  Upload(ctx, dA, A);
  Upload(ctx, dB, B);
  CheckRc(Dispatch<F>::lus(ctx, orientation == NORMAL ? 0 : 1, n, dA, n, dP, q, dB, n));
  CheckStatus(ctx, false);
  Download(B, dB);
}

// lu::SolveAfter(orientation, A, P, Q, B) (LU/SolveAfter.hpp:120-145).
template <typename F>
void SolveAfter(Orientation orientation, const Matrix<F>& A, const Permutation& P,
                const Permutation& Q, Matrix<F>& B) {
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  if (A.Height() != B.Height()) throw std::logic_error("A and B must be the same height");
  CallGuard guard;
  const Int n = A.Height(), q = B.Width();
  if (n == 0 || q == 0) return;
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)n * n), sb = Al(sizeof(F) * (size_t)n * q),
               sp = Al(sizeof(int) * n);
  char* base = Dev(sa + sb + 2 * sp);
  F* dA = reinterpret_cast<F*>(base);
  F* dB = reinterpret_cast<F*>(base + sa);
  int* dP = reinterpret_cast<int*>(base + sa + sb);
  int* dQ = reinterpret_cast<int*>(base + sa + sb + sp);
  const std::vector<int> pv = DevicePivots(P, n), qv = DevicePivots(Q, n);
  Check(cudaMemcpy(dP, pv.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "pivots");
  Check(cudaMemcpy(dQ, qv.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "pivots");
  Upload(ctx, dA, A);
  Upload(ctx, dB, B);
  CheckRc(Dispatch<F>::lufulls(ctx, orientation == NORMAL ? 0 : 1, n, dA, n, dP, dQ, q, dB, n));
  CheckStatus(ctx, false);
  Download(B, dB);
}
}  // namespace lu

// El::Cholesky(uplo, A, P) with diagonal pivoting (src/lapack_like/factor/
// Cholesky.cpp:44-52).
template <typename F>
void Cholesky(UpperOrLower uplo, Matrix<F>& A, Permutation& P) {
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  CallGuard guard;
  const Int n = A.Height();
  P.MakeIdentity(n);
  P.ReserveSwaps(n);
  if (n == 0) {
    P.SetSwapSequence(n, nullptr, 0);
    return;
  }
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)n * n);
  char* base = Dev(sa + Al(sizeof(int) * n));
  F* dA = reinterpret_cast<F*>(base);
  int* dP = reinterpret_cast<int*>(base + sa);
  Upload(ctx, dA, A);
  CheckRc(Dispatch<F>::cholpiv(ctx, uplo == UPPER ? 1 : 0, n, dA, n, dP));
  CheckStatus(ctx, true);
  Download(A, dA);
  std::vector<Int> p(n);
  Check(cudaMemcpy(p.data(), dP, sizeof(int) * n, cudaMemcpyDeviceToHost), "pivots");
  P.SetSwapSequence(n, p.data(), n);
}

template <typename F>
void Cholesky(UpperOrLower uplo, Matrix<F>& A) {
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  CallGuard guard;
  const Int n = A.Height();
  if (n == 0) return;
  ElGBContext ctx = Ctx();
  F* dA = reinterpret_cast<F*>(Dev(Al(sizeof(F) * (size_t)n * n)));
  Upload(ctx, dA, A);
  CheckRc(Dispatch<F>::chol(ctx, uplo == UPPER ? 1 : 0, n, dA, n, Blocksize()));
  int info = 0, err = 0;
  if (ElGBStatus(ctx, &info, &err) != 0) throw std::runtime_error("CUDA failure");
  Download(A, dA);
  if (err) throw std::runtime_error("device-side wait timed out");
  if (info) throw NonHPDMatrixException("A was not numerically HPD");
}

namespace cholesky {
template <typename F>
void SolveAfter(UpperOrLower uplo, Orientation orientation, const Matrix<F>& A, Matrix<F>& B) {
  (void)orientation;  // real scalars: Conjugate(B) is the identity
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  if (A.Height() != B.Height()) throw std::logic_error("A and B must be the same height");
  CallGuard guard;
  const Int n = A.Height(), q = B.Width();
  if (n == 0 || q == 0) return;
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)n * n);
  char* base = Dev(sa + Al(sizeof(F) * (size_t)n * q));
  F* dA = reinterpret_cast<F*>(base);
  F* dB = reinterpret_cast<F*>(base + sa);
  Upload(ctx, dA, A);
  Upload(ctx, dB, B);
  CheckRc(Dispatch<F>::chols(ctx, uplo == UPPER ? 1 : 0, n, dA, n, q, dB, n));
  CheckStatus(ctx, true);
  Download(B, dB);
}
}  // namespace cholesky

namespace cholesky {
// cholesky::SolveAfter(uplo, orientation, A, P, B) (Cholesky/SolveAfter.hpp:46-76);
// on real data the orientation changes nothing.
template <typename F>
void SolveAfter(UpperOrLower uplo, Orientation orientation, const Matrix<F>& A,
                const Permutation& P, Matrix<F>& B) {
  (void)orientation;
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  if (A.Height() != B.Height()) throw std::logic_error("A and B must be the same height");
  CallGuard guard;
  const Int n = A.Height(), q = B.Width();
  if (n == 0 || q == 0) return;
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)n * n), sb = Al(sizeof(F) * (size_t)n * q);
  char* base = Dev(sa + sb + Al(sizeof(int) * n));
  F* dA = reinterpret_cast<F*>(base);
  F* dB = reinterpret_cast<F*>(base + sa);
  int* dP = reinterpret_cast<int*>(base + sa + sb);
  const std::vector<int> pv = DevicePivots(P, n);
  Check(cudaMemcpy(dP, pv.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "pivots");
  Upload(ctx, dA, A);
  Upload(ctx, dB, B);
  CheckRc(Dispatch<F>::cholpivs(ctx, uplo == UPPER ? 1 : 0, n, dA, n, dP, q, dB, n));
  CheckStatus(ctx, true);
  Download(B, dB);
}
}  // namespace cholesky

template <typename F>
void LinearSolve(const Matrix<F>& A, Matrix<F>& B) {
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  if (A.Height() != B.Height()) throw std::logic_error("A and B must be the same height");
  CallGuard guard;
  const Int n = A.Height(), q = B.Width();
  if (n == 0) return;
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)n * n);
  char* base = Dev(sa + Al(sizeof(F) * (size_t)n * std::max(q, 1)));
  F* dA = reinterpret_cast<F*>(base);
  F* dB = reinterpret_cast<F*>(base + sa);
  Upload(ctx, dA, A);
  Upload(ctx, dB, B);
  CheckRc(Dispatch<F>::lin(ctx, n, dA, n, q, dB, n, Blocksize()));
  CheckStatus(ctx, false);
  Download(B, dB);
}

template <typename F>
void HPDSolve(UpperOrLower uplo, Orientation orientation, const Matrix<F>& A, Matrix<F>& B) {
  (void)orientation;
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  if (A.Height() != B.Height()) throw std::logic_error("A and B must be the same height");
  CallGuard guard;
  const Int n = A.Height(), q = B.Width();
  if (n == 0) return;
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(F) * (size_t)n * n);
  char* base = Dev(sa + Al(sizeof(F) * (size_t)n * std::max(q, 1)));
  F* dA = reinterpret_cast<F*>(base);
  F* dB = reinterpret_cast<F*>(base + sa);
  Upload(ctx, dA, A);
  Upload(ctx, dB, B);
  CheckRc(Dispatch<F>::hpd(ctx, uplo == UPPER ? 1 : 0, n, dA, n, q, dB, n, Blocksize()));
  CheckStatus(ctx, true);
  Download(B, dB);
}

void LastHostCallTimes(double* t) {
  std::lock_guard<std::mutex> lk(St().mu);
  for (int i = 0; i < 3; ++i) t[i] = St().last[i];
}

// Mixed-precision El::LinearSolve on host matrices (added form).
void LinearSolveMixed(const Matrix<double>& A, Matrix<double>& B, const ElGBRefineCtrl* ctrl,
                      ElGBRefineInfo* info) {
  if (A.Height() != A.Width()) throw std::logic_error("A must be square");
  if (A.Height() != B.Height()) throw std::logic_error("A and B must be the same height");
  CallGuard guard;
  const Int n = A.Height(), q = B.Width();
  if (n == 0 || q == 0) return;
  ElGBContext ctx = Ctx();
  const size_t sa = Al(sizeof(double) * (size_t)n * n), sb = Al(sizeof(double) * (size_t)n * q);
  char* base = Dev(sa + 2 * sb);
  double* dA = reinterpret_cast<double*>(base);
  double* dB = reinterpret_cast<double*>(base + sa);
  double* dX = reinterpret_cast<double*>(base + sa + sb);
  Upload(ctx, dA, A);
  Upload(ctx, dB, B);
  CheckRc(ElGBRefinedSolve_d(ctx, n, dA, n, q, dB, n, dX, n, ctrl, info));
  Check(cudaDeviceSynchronize(), "mixed solve");
  Download(B, dX);
}

// ---- matrix files: src/io/File.cpp:28-70 (extensions, DetectFormat),
// io/Write/Binary.hpp:17-37, io/Read/Binary.hpp:17-44, io/*/BinaryFlat.hpp ----
namespace {
const char* kExtensions[FileFormat_MAX] = {"",   "txt",  "m",  "bin", "dat", "bmp", "jpg",
                                           "jpeg", "mm", "png", "ppm", "xbm", "xpm"};

FileFormat DetectFormat(const std::string& filename) {
  const std::string ext = filename.substr(filename.find_last_of('.') + 1);
  for (int f = 1; f < FileFormat_MAX; ++f)
    if (ext == kExtensions[f]) return static_cast<FileFormat>(f);
  throw std::runtime_error("Did not detect file format");
}

long FileBytes(std::ifstream& f) {
  const auto pos = f.tellg();
  f.seekg(0, std::ios::end);
  const long bytes = static_cast<long>(f.tellg());
  f.seekg(pos);
  return bytes;
}
}  // namespace

template <typename T>
void Write(const Matrix<T>& A, const std::string& basename, FileFormat format,
           const std::string& title) {
  (void)title;  // the binary formats carry no title
  if (format != BINARY && format != BINARY_FLAT)
    throw std::logic_error("Format unsupported for writing a Matrix on this path");
  const std::string filename = basename + "." + kExtensions[format];
  std::ofstream f(filename, std::ios::binary);
  if (!f.is_open()) throw std::runtime_error("Could not open " + filename);
  if (format == BINARY) {
    const Int hw[2] = {A.Height(), A.Width()};
    f.write(reinterpret_cast<const char*>(hw), sizeof(hw));
  }
  for (Int j = 0; j < A.Width(); ++j)
    f.write(reinterpret_cast<const char*>(A.LockedBuffer(0, j)),
            static_cast<std::streamsize>(sizeof(T)) * A.Height());
  if (!f) throw std::runtime_error("Could not write " + filename);
}

template <typename T>
void Read(Matrix<T>& A, const std::string& filename, FileFormat format) {
  if (format == AUTO) format = DetectFormat(filename);
  if (format != BINARY && format != BINARY_FLAT)
    throw std::logic_error("Format unsupported for reading a Matrix");
  std::ifstream f(filename, std::ios::binary);
  if (!f.is_open()) throw std::runtime_error("Could not open " + filename);
  Int height = A.Height(), width = A.Width();  // BINARY_FLAT keeps A's shape
  long meta = 0;
  if (format == BINARY) {
    Int hw[2] = {0, 0};
    f.read(reinterpret_cast<char*>(hw), sizeof(hw));
    if (!f) throw std::runtime_error("Could not read the size of " + filename);
    height = hw[0];
    width = hw[1];
    meta = static_cast<long>(sizeof(hw));
  }
  if (height < 0 || width < 0) throw std::runtime_error("Invalid matrix size in " + filename);
  const long expect = meta + static_cast<long>(sizeof(T)) * height * width;
  if (FileBytes(f) != expect)
    throw std::runtime_error("Expected file to be " + std::to_string(expect) + " bytes");
  A.Resize(height, width);
  for (Int j = 0; j < width; ++j)
    f.read(reinterpret_cast<char*>(A.Buffer(0, j)),
           static_cast<std::streamsize>(sizeof(T)) * height);
  if (!f) throw std::runtime_error("Could not read " + filename);
}

template void Read<Int>(Matrix<Int>&, const std::string&, FileFormat);
template void Read<float>(Matrix<float>&, const std::string&, FileFormat);
template void Read<double>(Matrix<double>&, const std::string&, FileFormat);
template void Write<Int>(const Matrix<Int>&, const std::string&, FileFormat,
                         const std::string&);
template void Write<float>(const Matrix<float>&, const std::string&, FileFormat,
                           const std::string&);
template void Write<double>(const Matrix<double>&, const std::string&, FileFormat,
                            const std::string&);

#define EL_GB_PROTO(F)                                                                  \
  template void LU<F>(Matrix<F>&, Permutation&);                                        \
  template void LU<F>(Matrix<F>&);                                                      \
  template void LU<F>(Matrix<F>&, Permutation&, Permutation&);                          \
  template void Cholesky<F>(UpperOrLower, Matrix<F>&, Permutation&);                    \
  template void cholesky::SolveAfter<F>(UpperOrLower, Orientation, const Matrix<F>&,    \
                                        const Permutation&, Matrix<F>&);                \
  template void lu::SolveAfter<F>(Orientation, const Matrix<F>&, const Permutation&,    \
                                  const Permutation&, Matrix<F>&);                      \
  template void Inverse<F>(Matrix<F>&);                                                 \
  template F OneCondition<F>(const Matrix<F>&);                                         \
  template void lu::SolveAfter<F>(Orientation, const Matrix<F>&, const Permutation&,    \
                                  Matrix<F>&);                                          \
  template void Cholesky<F>(UpperOrLower, Matrix<F>&);                                  \
  template void cholesky::SolveAfter<F>(UpperOrLower, Orientation, const Matrix<F>&,    \
                                        Matrix<F>&);                                    \
  template void LinearSolve<F>(const Matrix<F>&, Matrix<F>&);                           \
  template void HPDSolve<F>(UpperOrLower, Orientation, const Matrix<F>&, Matrix<F>&);
EL_GB_PROTO(float)
EL_GB_PROTO(double)

}  // namespace El

// ===========================================================================
// C ABI (include/El_gb300.h), EL_TRY semantics
// ===========================================================================
#define EL_GB_TRY(payload)                                   \
  try {                                                      \
    payload;                                                 \
  } catch (std::bad_alloc&) {                                \
    return EL_ALLOC_ERROR;                                   \
  } catch (std::invalid_argument&) {                         \
    return EL_ARG_ERROR;                                     \
  } catch (std::logic_error&) {                              \
    return EL_LOGIC_ERROR;                                   \
  } catch (std::runtime_error&) {                            \
    return EL_RUNTIME_ERROR;                                 \
  } catch (std::exception&) {                                \
    return EL_ERROR;                                         \
  }                                                          \
  return EL_SUCCESS;

template <typename T>
static El::Matrix<T>* M(void* p) {
  return reinterpret_cast<El::Matrix<T>*>(p);
}
template <typename T>
static const El::Matrix<T>* CM(const void* p) {
  return reinterpret_cast<const El::Matrix<T>*>(p);
}
static El::Permutation* PP(void* p) { return reinterpret_cast<El::Permutation*>(p); }
static const El::Permutation* CP(const void* p) {
  return reinterpret_cast<const El::Permutation*>(p);
}

extern "C" {

const char* ElErrorString(ElError error) {
  switch (error) {
    case EL_SUCCESS: return "EL_SUCCESS";
    case EL_ALLOC_ERROR: return "EL_ALLOC_ERROR";
    case EL_OUT_OF_BOUNDS_ERROR: return "EL_OUT_OF_BOUNDS_ERROR";
    case EL_ARG_ERROR: return "EL_ARG_ERROR";
    case EL_LOGIC_ERROR: return "EL_LOGIC_ERROR";
    case EL_RUNTIME_ERROR: return "EL_RUNTIME_ERROR";
    default: return "EL_ERROR";
  }
}

#define EL_GB_MATRIX_IMPL(S, T)                                                          \
  ElError ElMatrixCreate_##S(ElMatrix_##S* A) {                                          \
    EL_GB_TRY(*A = reinterpret_cast<ElMatrix_##S>(new El::Matrix<T>()))                   \
  }                                                                                      \
  ElError ElMatrixDestroy_##S(ElConstMatrix_##S A) { EL_GB_TRY(delete CM<T>(A)) }        \
  ElError ElMatrixEmpty_##S(ElMatrix_##S A) { EL_GB_TRY(M<T>(A)->Empty()) }              \
  ElError ElMatrixResize_##S(ElMatrix_##S A, ElInt h, ElInt w) {                         \
    EL_GB_TRY(M<T>(A)->Resize(h, w))                                                     \
  }                                                                                      \
  ElError ElMatrixResizeWithLDim_##S(ElMatrix_##S A, ElInt h, ElInt w, ElInt ld) {       \
    EL_GB_TRY(M<T>(A)->Resize(h, w, ld))                                                 \
  }                                                                                      \
  ElError ElMatrixAttach_##S(ElMatrix_##S A, ElInt h, ElInt w, T* buf, ElInt ld) {       \
    EL_GB_TRY(M<T>(A)->Attach(h, w, buf, ld))                                            \
  }                                                                                      \
  ElError ElMatrixLockedAttach_##S(ElMatrix_##S A, ElInt h, ElInt w, const T* buf,       \
                                   ElInt ld) {                                           \
    EL_GB_TRY(M<T>(A)->LockedAttach(h, w, buf, ld))                                      \
  }                                                                                      \
  ElError ElMatrixHeight_##S(ElConstMatrix_##S A, ElInt* h) {                            \
    EL_GB_TRY(*h = CM<T>(A)->Height())                                                   \
  }                                                                                      \
  ElError ElMatrixWidth_##S(ElConstMatrix_##S A, ElInt* w) {                             \
    EL_GB_TRY(*w = CM<T>(A)->Width())                                                    \
  }                                                                                      \
  ElError ElMatrixLDim_##S(ElConstMatrix_##S A, ElInt* ld) {                             \
    EL_GB_TRY(*ld = CM<T>(A)->LDim())                                                    \
  }                                                                                      \
  ElError ElMatrixBuffer_##S(ElMatrix_##S A, T** buf) { EL_GB_TRY(*buf = M<T>(A)->Buffer()) } \
  ElError ElMatrixLockedBuffer_##S(ElConstMatrix_##S A, const T** buf) {                 \
    EL_GB_TRY(*buf = CM<T>(A)->LockedBuffer())                                           \
  }                                                                                      \
  ElError ElMatrixGet_##S(ElConstMatrix_##S A, ElInt i, ElInt j, T* val) {               \
    EL_GB_TRY(*val = CM<T>(A)->Get(i, j))                                                \
  }                                                                                      \
  ElError ElMatrixSet_##S(ElMatrix_##S A, ElInt i, ElInt j, T val) {                     \
    EL_GB_TRY(M<T>(A)->Set(i, j, val))                                                   \
  }                                                                                      \
  ElError ElView_##S(ElMatrix_##S A, ElMatrix_##S B, ElRange_i I, ElRange_i J) {         \
    EL_GB_TRY(El::View(*M<T>(A), *M<T>(B), El::IR(I.beg, I.end), El::IR(J.beg, J.end)))  \
  }                                                                                      \
  ElError ElLockedView_##S(ElMatrix_##S A, ElConstMatrix_##S B, ElRange_i I,             \
                           ElRange_i J) {                                                \
    EL_GB_TRY(El::LockedView(*M<T>(A), *CM<T>(B), El::IR(I.beg, I.end),                  \
                             El::IR(J.beg, J.end)))                                      \
  }
EL_GB_MATRIX_IMPL(i, ElInt)
EL_GB_MATRIX_IMPL(s, float)
EL_GB_MATRIX_IMPL(d, double)

ElError ElPermutationCreate(ElPermutation* P) {
  EL_GB_TRY(*P = reinterpret_cast<ElPermutation>(new El::Permutation()))
}
ElError ElPermutationDestroy(ElConstPermutation P) { EL_GB_TRY(delete CP(P)) }
ElError ElPermutationEmpty(ElPermutation P) { EL_GB_TRY(PP(P)->Empty()) }
ElError ElPermutationMakeIdentity(ElPermutation P, ElInt size) {
  EL_GB_TRY(PP(P)->MakeIdentity(size))
}
ElError ElPermutationReserveSwaps(ElPermutation P, ElInt maxSwaps) {
  EL_GB_TRY(PP(P)->ReserveSwaps(maxSwaps))
}
ElError ElPermutationSwap(ElPermutation P, ElInt origin, ElInt dest) {
  EL_GB_TRY(PP(P)->Swap(origin, dest))
}
ElError ElPermutationSwapSequence(ElPermutation P, ElConstPermutation PAppend, ElInt offset) {
  EL_GB_TRY(PP(P)->SwapSequence(*CP(PAppend), offset))
}
ElError ElPermutationHeight(ElConstPermutation P, ElInt* h) { EL_GB_TRY(*h = CP(P)->Height()) }
ElError ElPermutationWidth(ElConstPermutation P, ElInt* w) { EL_GB_TRY(*w = CP(P)->Width()) }
ElError ElPermutationParity(ElConstPermutation P, bool* parity) {
  EL_GB_TRY(*parity = CP(P)->Parity())
}
ElError ElPermutationIsSwapSequence(ElConstPermutation P, bool* isSwap) {
  EL_GB_TRY(*isSwap = CP(P)->IsSwapSequence())
}
ElError ElPermutationIsImplicitSwapSequence(ElConstPermutation P, bool* isImplicit) {
  EL_GB_TRY(*isImplicit = CP(P)->IsImplicitSwapSequence())
}
ElError ElPermutationPermuteRows_s(ElConstPermutation P, ElMatrix_s A, ElInt offset) {
  EL_GB_TRY(CP(P)->PermuteRows(*M<float>(A), offset))
}
ElError ElPermutationPermuteRows_d(ElConstPermutation P, ElMatrix_d A, ElInt offset) {
  EL_GB_TRY(CP(P)->PermuteRows(*M<double>(A), offset))
}
ElError ElPermutationExplicitVector(ElConstPermutation P, ElMatrix_i pVec) {
  EL_GB_TRY(CP(P)->ExplicitVector(*M<El::Int>(pVec)))
}

ElError ElBlocksize(ElInt* blocksize) { EL_GB_TRY(*blocksize = El::Blocksize()) }
ElError ElSetBlocksize(ElInt blocksize) { EL_GB_TRY(El::SetBlocksize(blocksize)) }
ElError ElPushBlocksizeStack(ElInt blocksize) { EL_GB_TRY(El::PushBlocksizeStack(blocksize)) }
ElError ElPopBlocksizeStack(void) { EL_GB_TRY(El::PopBlocksizeStack()) }

static El::Orientation Or(ElOrientation o) {
  return o == EL_NORMAL ? El::NORMAL : (o == EL_TRANSPOSE ? El::TRANSPOSE : El::ADJOINT);
}
static El::UpperOrLower Ul(ElUpperOrLower u) { return u == EL_UPPER ? El::UPPER : El::LOWER; }

ElError ElLUPartialPiv_s(ElMatrix_s A, ElPermutation P) { EL_GB_TRY(El::LU(*M<float>(A), *PP(P))) }
ElError ElLUPartialPiv_d(ElMatrix_d A, ElPermutation P) {
  EL_GB_TRY(El::LU(*M<double>(A), *PP(P)))
}
#define EL_GB_IO(S, T)                                                                    \
  ElError ElRead_##S(ElMatrix_##S A, const char* filename, ElFileFormat format) {          \
    if (!A || !filename) return EL_ARG_ERROR;                                              \
    EL_GB_TRY(El::Read(*M<T>(A), filename, static_cast<El::FileFormat>(format)))          \
  }                                                                                        \
  ElError ElWrite_##S(ElConstMatrix_##S A, const char* basename, ElFileFormat format,      \
                      const char* title) {                                                 \
    if (!A || !basename) return EL_ARG_ERROR;                                              \
    EL_GB_TRY(El::Write(*CM<T>(A), basename, static_cast<El::FileFormat>(format),          \
                        title ? title : ""))                                               \
  }
EL_GB_IO(i, El::Int)
EL_GB_IO(s, float)
EL_GB_IO(d, double)
ElError ElLUFullPiv_s(ElMatrix_s A, ElPermutation P, ElPermutation Q) {
  EL_GB_TRY(El::LU(*M<float>(A), *PP(P), *PP(Q)))
}
ElError ElLUFullPiv_d(ElMatrix_d A, ElPermutation P, ElPermutation Q) {
  EL_GB_TRY(El::LU(*M<double>(A), *PP(P), *PP(Q)))
}
ElError ElSolveAfterLUFullPiv_s(ElOrientation o, ElConstMatrix_s A, ElConstPermutation P,
                                ElConstPermutation Q, ElMatrix_s B) {
  EL_GB_TRY(El::lu::SolveAfter(static_cast<El::Orientation>(o), *CM<float>(A), *CP(P), *CP(Q),
                               *M<float>(B)))
}
ElError ElSolveAfterLUFullPiv_d(ElOrientation o, ElConstMatrix_d A, ElConstPermutation P,
                                ElConstPermutation Q, ElMatrix_d B) {
  EL_GB_TRY(El::lu::SolveAfter(static_cast<El::Orientation>(o), *CM<double>(A), *CP(P),
                               *CP(Q), *M<double>(B)))
}
ElError ElCholeskyPiv_s(ElUpperOrLower u, ElMatrix_s A, ElPermutation P) {
  EL_GB_TRY(El::Cholesky(Ul(u), *M<float>(A), *PP(P)))
}
ElError ElCholeskyPiv_d(ElUpperOrLower u, ElMatrix_d A, ElPermutation P) {
  EL_GB_TRY(El::Cholesky(Ul(u), *M<double>(A), *PP(P)))
}
ElError ElSolveAfterCholeskyPiv_s(ElUpperOrLower u, ElOrientation o, ElConstMatrix_s A,
                                  ElConstPermutation P, ElMatrix_s B) {
  EL_GB_TRY(El::cholesky::SolveAfter(Ul(u), Or(o), *CM<float>(A), *CP(P), *M<float>(B)))
}
ElError ElSolveAfterCholeskyPiv_d(ElUpperOrLower u, ElOrientation o, ElConstMatrix_d A,
                                  ElConstPermutation P, ElMatrix_d B) {
  EL_GB_TRY(El::cholesky::SolveAfter(Ul(u), Or(o), *CM<double>(A), *CP(P), *M<double>(B)))
}
ElError ElLU_s(ElMatrix_s A) { EL_GB_TRY(El::LU(*M<float>(A))) }
ElError ElLU_d(ElMatrix_d A) { EL_GB_TRY(El::LU(*M<double>(A))) }
ElError ElInverse_s(ElMatrix_s A) { EL_GB_TRY(El::Inverse(*M<float>(A))) }
ElError ElInverse_d(ElMatrix_d A) { EL_GB_TRY(El::Inverse(*M<double>(A))) }
ElError ElOneCondition_s(ElConstMatrix_s A, float* cond) {
  if (!cond) return EL_ARG_ERROR;
  EL_GB_TRY(*cond = El::OneCondition(*CM<float>(A)))
}
ElError ElOneCondition_d(ElConstMatrix_d A, double* cond) {
  if (!cond) return EL_ARG_ERROR;
  EL_GB_TRY(*cond = El::OneCondition(*CM<double>(A)))
}
ElError ElSolveAfterLUPartialPiv_s(ElOrientation o, ElConstMatrix_s A, ElConstPermutation P,
                                   ElMatrix_s B) {
  EL_GB_TRY(El::lu::SolveAfter(Or(o), *CM<float>(A), *CP(P), *M<float>(B)))
}
ElError ElSolveAfterLUPartialPiv_d(ElOrientation o, ElConstMatrix_d A, ElConstPermutation P,
                                   ElMatrix_d B) {
  EL_GB_TRY(El::lu::SolveAfter(Or(o), *CM<double>(A), *CP(P), *M<double>(B)))
}
ElError ElCholesky_s(ElUpperOrLower u, ElMatrix_s A) { EL_GB_TRY(El::Cholesky(Ul(u), *M<float>(A))) }
ElError ElCholesky_d(ElUpperOrLower u, ElMatrix_d A) {
  EL_GB_TRY(El::Cholesky(Ul(u), *M<double>(A)))
}
ElError ElSolveAfterCholesky_s(ElUpperOrLower u, ElOrientation o, ElConstMatrix_s A,
                               ElMatrix_s B) {
  EL_GB_TRY(El::cholesky::SolveAfter(Ul(u), Or(o), *CM<float>(A), *M<float>(B)))
}
ElError ElSolveAfterCholesky_d(ElUpperOrLower u, ElOrientation o, ElConstMatrix_d A,
                               ElMatrix_d B) {
  EL_GB_TRY(El::cholesky::SolveAfter(Ul(u), Or(o), *CM<double>(A), *M<double>(B)))
}
ElError ElLinearSolve_s(ElConstMatrix_s A, ElMatrix_s B) {
  EL_GB_TRY(El::LinearSolve(*CM<float>(A), *M<float>(B)))
}
ElError ElLinearSolve_d(ElConstMatrix_d A, ElMatrix_d B) {
  EL_GB_TRY(El::LinearSolve(*CM<double>(A), *M<double>(B)))
}
ElError ElLinearSolveMixed_d(ElConstMatrix_d A, ElMatrix_d B, const ElGBRefineCtrl* ctrl,
                             ElGBRefineInfo* info) {
  EL_GB_TRY(El::LinearSolveMixed(*CM<double>(A), *M<double>(B), ctrl, info))
}
// Host buffers: anonymous mappings registered with the driver, by length.
static std::mutex g_host_mu;
static std::unordered_map<void*, size_t>& HostMaps() {
  static std::unordered_map<void*, size_t> m;
  return m;
}

ElError ElGBHostAlloc(size_t bytes, void** ptr) {
  if (!ptr) return EL_ARG_ERROR;
  *ptr = nullptr;
  if (bytes == 0) return EL_SUCCESS;
  const size_t align = size_t(2) << 20;
  const size_t len = (bytes + align - 1) / align * align;
  void* p = mmap(nullptr, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (p == MAP_FAILED) return EL_ALLOC_ERROR;
#ifdef MADV_HUGEPAGE
  madvise(p, len, MADV_HUGEPAGE);  // advice only: without it the pages stay small
#endif
  if (cudaHostRegister(p, len, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    munmap(p, len);
    return EL_RUNTIME_ERROR;
  }
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    HostMaps()[p] = len;
  }
  *ptr = p;
  return EL_SUCCESS;
}

ElError ElGBHostFree(void* ptr) {
  if (!ptr) return EL_SUCCESS;
  size_t len = 0;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = HostMaps().find(ptr);
    if (it == HostMaps().end()) return EL_LOGIC_ERROR;
    len = it->second;
    HostMaps().erase(it);
  }
  cudaHostUnregister(ptr);
  cudaGetLastError();
  munmap(ptr, len);
  return EL_SUCCESS;
}

ElError ElGBLastHostCallTimes(double* upload_ms, double* compute_ms, double* download_ms) {
  double t[3];
  El::LastHostCallTimes(t);
  if (upload_ms) *upload_ms = t[0];
  if (compute_ms) *compute_ms = t[1];
  if (download_ms) *download_ms = t[2];
  return EL_SUCCESS;
}
ElError ElHPDSolve_s(ElUpperOrLower u, ElOrientation o, ElConstMatrix_s A, ElMatrix_s B) {
  EL_GB_TRY(El::HPDSolve(Ul(u), Or(o), *CM<float>(A), *M<float>(B)))
}
ElError ElHPDSolve_d(ElUpperOrLower u, ElOrientation o, ElConstMatrix_d A, ElMatrix_d B) {
  EL_GB_TRY(El::HPDSolve(Ul(u), Or(o), *CM<double>(A), *M<double>(B)))
}

}  // extern "C"
