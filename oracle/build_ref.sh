#!/usr/bin/env bash
# Builds the reference's OWN sequential factor-and-solve path (Elemental
# El::LU with and without pivoting / lu::SolveAfter / El::Cholesky /
# cholesky::SolveAfter / El::LinearSolve / El::HPDSolve / El::Inverse /
# El::OneCondition) from its sources, in place, into
# oracle/_ref/elref.  Test infrastructure only: the product never links it.
#
# Nothing is copied out of the reference tree.  The recipe:
#   1. El/config.h generated from the reference's cmake/configure_files/
#      config.h.in (the #cmakedefine switches a sequential, MPI-less build
#      needs are turned on, the rest off);
#   2. the single-rank stub <mpi.h> in oracle/stub/;
#   3. g++ on the reference's own translation units under src/core,
#      src/blas_like, src/lapack_like/{perm,props}, src/matrices, plus
#      LU.cpp, Cholesky.cpp, Linear.cpp, HPD.cpp and the general and
#      triangular Inverse (funcs/Inverse/{General,Triangular}.cpp, which
#      OneCondition in props calls) and the matrix file reader / writer
#      (io/{File,Read,Write}.cpp);
#   4. the BLAS names Elemental calls (bare, e.g. `dgemm`; no-suffix mangling
#      include/El/core/imports/blas.hpp:29-41) renamed in the objects to the
#      symbols of SciPy's bundled OpenBLAS (`scipy_dgemm_`), which is linked;
#   5. an executable harness (oracle/ref_harness.cpp) linked with unresolved
#      MPI / METIS / distributed symbols left undefined: the sequential path
#      never reaches them.
# Usage: oracle/build_ref.sh [reference-root]   (default /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${ELEMENTAL_REF:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/lapack_like/factor/LU.cpp" ]; then
  echo "build_ref: reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/include/El" "$OUT/obj"

# 1. config.h
ON="EL_RELEASE BUILD_SHARED_LIBS EL_HAVE_PRETTY_FUNCTION EL_HAVE_CXX11RANDOM
EL_HAVE_STEADYCLOCK EL_HAVE_NOEXCEPT EL_HAVE_METIS EL_AVOID_COMPLEX_MPI
EL_USE_CUSTOM_ALLTOALLV EL_HAVE_MPI_REDUCE_SCATTER_BLOCK EL_HAVE_MPI_LONG_LONG
EL_HAVE_MPI_INIT_THREAD EL_HAVE_MPI_QUERY_THREAD
EL_HAVE_MPI_COMM_SET_ERRHANDLER"
SEDS=()
for d in $ON; do SEDS+=(-e "s/^#cmakedefine $d\$/#define $d/"); done
sed "${SEDS[@]}" \
    -e 's/^#cmakedefine \([A-Za-z0-9_]*\)$/\/* #undef \1 *\//' \
    -e 's/@EL_FORT_LOGICAL@/int/' -e 's/@EL_FORT_TRUE@/1/' \
    -e 's/@EL_FORT_FALSE@/0/' -e 's/@EL_RESTRICT@/__restrict__/' \
    -e 's/@[A-Za-z0-9_]*@//g' \
    "$REF/cmake/configure_files/config.h.in" > "$OUT/include/El/config.h.new"
if ! cmp -s "$OUT/include/El/config.h.new" "$OUT/include/El/config.h"; then
  mv "$OUT/include/El/config.h.new" "$OUT/include/El/config.h"
else
  rm -f "$OUT/include/El/config.h.new"
fi

# 3. translation units
TUS=$(cd "$REF" && { find src/core src/blas_like src/lapack_like/perm \
        src/lapack_like/props src/matrices -name '*.cpp' \
        ! -name '*-C.cpp' ! -name 'qt5.cpp';
      echo src/lapack_like/factor/LU.cpp;
      echo src/lapack_like/factor/Cholesky.cpp;
      echo src/lapack_like/solve/Linear.cpp;
      echo src/lapack_like/solve/HPD.cpp;
      echo src/lapack_like/funcs/Inverse/General.cpp;
      echo src/lapack_like/funcs/Inverse/Triangular.cpp;
      echo src/io/File.cpp; echo src/io/Read.cpp; echo src/io/Write.cpp; } | sort)
CXXFLAGS="-std=c++14 -O2 -fPIC -w -I$OUT/include -I$HERE/stub -I$REF/include
 -I$REF/external/suite_sparse/include -I$REF/external/pmrrr/include"
export REF OUT CXXFLAGS
echo "$TUS" | xargs -P "$(nproc)" -I{} bash -c '
  o="$OUT/obj/$(echo {} | tr / _).o"
  if [ ! -f "$o" ] || [ "$REF/{}" -nt "$o" ]; then
    g++ $CXXFLAGS -c "$REF/{}" -o "$o"
  fi'

# 4. BLAS renaming onto SciPy's OpenBLAS (LP64, matches the reference's
#    default 32-bit BlasInt)
BLAS_SO=$(python3 -c 'import scipy,os,glob;print(sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__),"..","scipy.libs","libscipy_openblas-*.so")))[0])')
BLAS_SO=$(readlink -f "$BLAS_SO")
nm -D --defined-only "$BLAS_SO" | awk '{print $3}' \
  | sed -n 's/^scipy_\([a-z0-9]*\)_$/\1/p' | sort -u > "$OUT/blas_names.txt"
nm -u "$OUT"/obj/*.o | awk '{print $2}' | sort -u > "$OUT/undef.txt"
comm -12 "$OUT/blas_names.txt" "$OUT/undef.txt" \
  | awk '{print $1" scipy_"$1"_"}' > "$OUT/redefine.txt"
mkdir -p "$OUT/objr"
for o in "$OUT"/obj/*.o; do
  r="$OUT/objr/$(basename "$o")"
  if [ ! -f "$r" ] || [ "$o" -nt "$r" ] || [ "$OUT/redefine.txt" -nt "$r" ]; then
    objcopy --redefine-syms="$OUT/redefine.txt" "$o" "$r"
  fi
done

# 5. harness
g++ $CXXFLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o"
objcopy --redefine-syms="$OUT/redefine.txt" "$OUT/ref_harness.o"
g++ -o "$OUT/elref" "$OUT/ref_harness.o" "$OUT"/objr/*.o "$BLAS_SO" \
    -Wl,-rpath,"$(dirname "$BLAS_SO")" -Wl,--unresolved-symbols=ignore-all \
    -lpthread
echo "build_ref: built $OUT/elref"
