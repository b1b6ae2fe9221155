"""Generates the golden fixtures in this folder by running the REFERENCE's own
sequential path (Elemental's El::LU with and without pivoting,
lu::SolveAfter, El::Cholesky, cholesky::SolveAfter, El::LinearSolve,
El::HPDSolve, El::Inverse, El::OneCondition, El::Write), compiled from its
sources into oracle/_ref/elref by oracle/build_ref.sh.

Run (where the reference tree is present):
    oracle/build_ref.sh && python tests/golden/gen_golden.py [name-prefix ...]

Each fixture is an .npz with the inputs (or, for the large config-1 case, the
seed plus a SHA-256 of the regenerated input), the blocksize, the
reference's outputs and its exit status.  The reference has no golden vectors
of its own (its tests check residual ratios only), so these pin the parity of
the oracle restatement and of the GPU path.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from elemental_gb300 import matrices as mats  # noqa: E402
from oracle import oracle as O  # noqa: E402

F64, I32 = np.float64, np.int32


def sha(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def save(name, **kw):
    # optional arguments: only fixtures whose names start with one of them
    if len(sys.argv) > 1 and not any(name.startswith(p) for p in sys.argv[1:]):
        return
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **kw)
    print("wrote", name)


def lu_case(name, A, nb, dtype=F64, store_input=True):
    st, out = O.ref_run("lu", nb=nb, dtype=dtype, inputs=[A], out_dtypes=[dtype, I32])
    kw = dict(op="lu", nb=nb, status=st, dtype=np.dtype(dtype).name)
    if store_input:
        kw["A"] = A.astype(dtype)
    if st == 0:
        kw["LU"], kw["piv"] = out[0], out[1].ravel()
    save(name, **kw)


def main():
    if not O.have_reference():
        sys.exit("oracle/_ref/elref missing: run oracle/build_ref.sh first")
    s = mats.BASE_SEED
    # LU (tests/lapack_like/LU.cpp defaults: --height 100 --nb 96)
    lu_case("lu_100_nb96", mats.gaussian(100, 100, s + 100), 96)
    lu_case("lu_gepp_growth_100_nb96", mats.gepp_growth(100), 96)
    lu_case("lu_129_nb32", mats.gaussian(129, 129, s + 129), 32)
    lu_case("lu_150x100_nb32", mats.gaussian(150, 100, s + 150), 32)
    lu_case("lu_100x150_nb32", mats.gaussian(100, 150, s + 151), 32)
    lu_case("lu_33_nb32", mats.gaussian(33, 33, s + 33), 32)
    lu_case("lu_1_nb128", mats.gaussian(1, 1, s + 1), 128)
    Z = mats.gaussian(50, 50, s + 50)
    Z[:, 17] = 0.0
    lu_case("lu_singular_50_nb16", Z, 16)
    lu_case("lu_s_100_nb96", mats.gaussian(100, 100, s + 101), 96, dtype=np.float32)

    # lu::SolveAfter NORMAL / TRANSPOSE
    for o in ("N", "T"):
        A = mats.gaussian(120, 120, s + 201)
        B = mats.gaussian(120, 3, s + 202)
        st, out = O.ref_run("lusolve", o, nb=32, inputs=[A, B], out_dtypes=[F64, I32, F64])
        save(f"lusolve_{o}_120_nb32", op="lusolve", orient=o, nb=32, status=st, A=A, B=B,
             LU=out[0], piv=out[1].ravel(), X=out[2])

    # Cholesky (tests/lapack_like/Cholesky.cpp: HermitianUniformSpectrum(m,1e-9,10), m 100, nb 96)
    H = mats.hermitian_uniform_spectrum(100, 1e-9, 10.0, s + 400)
    S = mats.spd(120, s + 401)
    for u in ("L", "U"):
        st, out = O.ref_run("chol", u, nb=96, inputs=[H], out_dtypes=[F64])
        save(f"chol_{u}_hus100_nb96", op="chol", uplo=u, nb=96, status=st, A=H, C=out[0])
        B = mats.gaussian(120, 4, s + 402)
        st, out = O.ref_run("cholsolve", u, nb=32, inputs=[S, B], out_dtypes=[F64, F64])
        save(f"cholsolve_{u}_spd120_nb32", op="cholsolve", uplo=u, nb=32, status=st, A=S, B=B,
             C=out[0], X=out[1])
        st, out = O.ref_run("hpdsolve", u, nb=32, inputs=[S, B], out_dtypes=[F64])
        save(f"hpdsolve_{u}_spd120_nb32", op="hpdsolve", uplo=u, nb=32, status=st, A=S, B=B,
             X=out[0])
    G = mats.gaussian(60, 60, s + 403)
    st, _ = O.ref_run("chol", "L", nb=16, inputs=[G], out_dtypes=[F64])
    save("chol_nonhpd_60_nb16", op="chol", uplo="L", nb=16, status=st, A=G)

    # El::Cholesky(uplo, A, P) with diagonal pivoting (Cholesky.cpp:44-52 ->
    # Cholesky/Pivoted{Lower,Upper}Variant3.hpp: lazy panels of Blocksize()
    # columns, the largest updated diagonal entry first -- the first on ties)
    # and cholesky::SolveAfter(uplo, orientation, A, P, B) (SolveAfter.hpp:46-76)
    Sp = mats.spd(90, s + 650)
    Cr = mats.spd(70, s + 651)
    dg = np.sqrt(np.diag(Cr))
    Cr = Cr / dg[:, None] / dg[None, :]
    np.fill_diagonal(Cr, 1.0)  # a correlation matrix: every diagonal entry ties
    # (the reference's PivotedLowerPanel reads X(i, -1) of an empty view at
    # each panel's first column -- memory before the buffer; with 8 or 16
    # column panels on this correlation matrix that read is non-zero on later
    # panels and changes the pivots, so the fixtures use panel widths where it
    # is not)
    for u in ("L", "U"):
        for name, M, nb in ((f"cholpiv_{u}_spd90_nb32", Sp, 32),
                            (f"cholpiv_{u}_corr70_nb32", Cr, 32)):
            st, out = O.ref_run("cholpiv", u, nb=nb, inputs=[M], out_dtypes=[F64, I32])
            save(name, op="cholpiv", uplo=u, nb=nb, status=st, A=M, C=out[0], piv=out[1].ravel())
        B = mats.gaussian(90, 3, s + 652)
        st, out = O.ref_run("cholpivsolve", u, nb=32, inputs=[Sp, B],
                            out_dtypes=[F64, I32, F64])
        save(f"cholpivsolve_{u}_spd90_nb32", op="cholpivsolve", uplo=u, nb=32, status=st, A=Sp,
             B=B, C=out[0], piv=out[1].ravel(), X=out[2])

    # El::LinearSolve
    A = mats.gaussian(120, 120, s + 500)
    B = mats.gaussian(120, 5, s + 501)
    st, out = O.ref_run("linsolve", nb=32, inputs=[A, B], out_dtypes=[F64])
    save("linsolve_120_nb32", op="linsolve", nb=32, status=st, A=A, B=B, X=out[0])

    # El::LU without pivoting (src/lapack_like/factor/LU.cpp:21-44): square,
    # wide and tall, diagonally dominant (stable without pivoting), and an
    # exact zero pivot (lu::Unb throws SingularMatrixException)
    D = mats.gaussian(100, 100, s + 600) + 100.0 * np.eye(100)
    for name, M in (("lunopiv_100_nb32", D),
                    ("lunopiv_90x130_nb32", mats.gaussian(90, 130, s + 601)
                     + np.hstack([90.0 * np.eye(90), np.zeros((90, 40))])),
                    ("lunopiv_130x90_nb32", mats.gaussian(130, 90, s + 602)
                     + np.vstack([90.0 * np.eye(90), np.zeros((40, 90))]))):
        st, out = O.ref_run("lunopiv", nb=32, inputs=[M], out_dtypes=[F64])
        save(name, op="lunopiv", nb=32, status=st, A=M, LU=out[0])
    Zp = D.copy()
    Zp[40, 40] = 0.0
    Zp[40, :] = 0.0
    st, _ = O.ref_run("lunopiv", nb=32, inputs=[Zp], out_dtypes=[F64])
    save("lunopiv_singular_100_nb32", op="lunopiv", nb=32, status=st, A=Zp)

    # El::LU(A, P, Q) with full pivoting (LU.cpp:145-152 -> LU/Full.hpp:15-59:
    # MaxAbsLoc over the trailing block, row and column swap, scale, rank-1
    # update) and lu::SolveAfter(orientation, A, P, Q, B) (LU/SolveAfter.hpp)
    for name, M in (("lufull_60", mats.gaussian(60, 60, s + 630)),
                    ("lufull_70x45", mats.gaussian(70, 45, s + 631)),
                    ("lufull_45x70", mats.gaussian(45, 70, s + 632))):
        st, out = O.ref_run("lufull", nb=32, inputs=[M], out_dtypes=[F64, I32, I32])
        save(name, op="lufull", nb=32, status=st, A=M, LU=out[0], p=out[1].ravel(),
             q=out[2].ravel())
    st, _ = O.ref_run("lufull", nb=32, inputs=[np.zeros((30, 30))], out_dtypes=[F64, I32, I32])
    save("lufull_zero_30", op="lufull", nb=32, status=st, A=np.zeros((30, 30)))
    M = mats.gaussian(16, 16, s + 635)
    M.ravel()[::7] = np.round(M.ravel()[::7])
    M[3, 5] = M[7, 2] = 4.0  # an exact tie for the first pivot: first in column order wins
    st, out = O.ref_run("lufull", nb=32, inputs=[M], out_dtypes=[F64, I32, I32])
    save("lufull_tie_16", op="lufull", nb=32, status=st, A=M, LU=out[0], p=out[1].ravel(),
         q=out[2].ravel())
    for o in ("N", "T"):
        A = mats.gaussian(64, 64, s + 640)
        B = mats.gaussian(64, 3, s + 641)
        st, out = O.ref_run("lufullsolve", o, nb=32, inputs=[A, B],
                            out_dtypes=[F64, I32, I32, F64])
        save(f"lufullsolve_{o}_64", op="lufullsolve", orient=o, nb=32, status=st, A=A, B=B,
             LU=out[0], p=out[1].ravel(), q=out[2].ravel(), X=out[3])

    # El::Inverse (funcs/Inverse/General/LUPartialPiv.hpp: LU, TriangularInverse,
    # the backward sweep against L, InversePermuteCols) and El::OneCondition
    # (props/Condition/One.cpp: ||A||_1 ||inv(A)||_1, +inf when singular)
    for name, M, nb in (("inverse_100_nb32", mats.gaussian(100, 100, s + 610), 32),
                        ("inverse_129_nb96", mats.gaussian(129, 129, s + 611), 96),
                        ("inverse_haar_k1e6_80_nb16", mats.conditioned(80, 1e6, s + 612), 16)):
        st, out = O.ref_run("inverse", nb=nb, inputs=[M], out_dtypes=[F64])
        save(name, op="inverse", nb=nb, status=st, A=M, Ainv=out[0])
    M = mats.gaussian(64, 64, s + 613)
    st, out = O.ref_run("inverse", nb=32, dtype=np.float32, inputs=[M], out_dtypes=[np.float32])
    save("inverse_s_64_nb32", op="inverse", nb=32, status=st, dtype="float32",
         A=M.astype(np.float32), Ainv=out[0])
    Zi = mats.gaussian(50, 50, s + 614)
    Zi[:, 7] = 0.0
    st, _ = O.ref_run("inverse", nb=16, inputs=[Zi], out_dtypes=[F64])
    save("inverse_singular_50_nb16", op="inverse", nb=16, status=st, A=Zi)
    for name, M in (("onecond_haar_k1e4_80", mats.conditioned(80, 1e4, s + 620)),
                    ("onecond_gauss_120", mats.gaussian(120, 120, s + 621)),
                    ("onecond_singular_50", Zi)):
        st, out = O.ref_run("onecond", nb=32, inputs=[M], out_dtypes=[F64])
        save(name, op="onecond", nb=32, status=st, A=M, cond=out[0].ravel()[0])

    # El::Write (src/io/Write/Binary.hpp, BinaryFlat.hpp): the reference's
    # file bytes for BINARY and BINARY_FLAT, FP64 and FP32
    import tempfile
    for fmt, ext in (("bin", "bin"), ("dat", "dat")):
        for dt, sfx in ((F64, "d"), (np.float32, "s")):
            M = mats.gaussian(7, 5, s + 700).astype(dt)
            with tempfile.TemporaryDirectory() as d:
                base = os.path.join(d, "m")
                st, _ = O.ref_run("write", fmt, base, nb=32, dtype=dt, inputs=[M], out_dtypes=[])
                with open(base + "." + ext, "rb") as f:
                    raw = np.frombuffer(f.read(), dtype=np.uint8)
            save(f"io_write_{fmt}_{sfx}_7x5", op="write", fmt=fmt, status=st, A=M, raw=raw,
                 dtype=np.dtype(dt).name)

    # Config 1: n = 1024, 1 RHS, iid N(0,1), nb = 128 (the default blocksize)
    n = 1024
    A = mats.gaussian(n, n, s + 1)
    b = mats.gaussian(n, 1, s + 1001)
    st, out = O.ref_run("lusolve", "N", nb=128, inputs=[A, b], out_dtypes=[F64, I32, F64])
    berr = O.backward_error(A, out[2], b)
    save("cfg1_lusolve_1024_nb128", op="lusolve", orient="N", nb=128, status=st, n=n,
         seed_A=s + 1, seed_b=s + 1001, sha_A=sha(A), sha_b=sha(b), piv=out[1].ravel(),
         X=out[2], berr=berr, LU_fro=np.linalg.norm(out[0]), LU_diag=np.diag(out[0]).copy())


if __name__ == "__main__":
    main()
