"""Build the reference's own QR path into oracle/_ref/libcandmc_ref.so.

TEST INFRASTRUCTURE ONLY.  The reference (solomonik/CANDMC) is plain C++ over
MPI and LAPACK.  This recipe compiles its QR sources unmodified, where they
lie in the reference checkout, with the reference's default optimisation
flags (-O3 -fopenmp, configure:179), against two project-written adapters:

  oracle/ref_shim/mpi.h        a single-rank MPI (the image has no MPI);
  LAPACK/BLAS                  scipy's bundled OpenBLAS (LP64, symbols
                               prefixed `scipy_`): each Fortran name the
                               reference's wrappers call (alg/shared/
                               lapack.cxx:40-70 with FTN_UNDERSCORE) is renamed
                               on the command line to its `scipy_` entry point.

plus oracle/ref_shim/ref_driver.cxx, C entry points that build the 1 x 1
grid and call one reference function each.  The output goes only to
oracle/_ref/ (git-ignored).  The reference's own configure/Makefiles are not
used.  The checkout is looked up in $CANDMC_REFERENCE, else /root/reference;
without it the build is skipped (it exists only where the reference does).

    python -m oracle.build_ref [--force]
"""
import glob
import os
import subprocess
import sys
import concurrent.futures

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libcandmc_ref.so")

# reference sources of the QR hot path and the shared layer they need
SOURCES = [
    "alg/shared/lapack.cxx",
    "alg/shared/util.cxx",
    "alg/shared/timer.cxx",
    "alg/QR/tsqr/bitree_tsqr.cxx",
    "alg/QR/tsqr/construct_tsqr_Q.cxx",
    "alg/QR/tsqr/apply_tsqr_QT.cxx",
    "alg/QR/hh_recon/hh_recon.cxx",
    "alg/QR/hh_recon/yamamoto.cxx",
    "alg/QR/qr_2d/qr_2d.cxx",
    "alg/QR/qr_2d/qr_y2d.cxx",
]

# Fortran BLAS/LAPACK names reached through alg/shared/lapack.cxx
FORTRAN = ["dgemm", "zgemm", "daxpy", "zaxpy", "dcopy", "zcopy", "dscal", "zscal", "ddot", "dgetrf",
           "dtrsm", "dsyrk", "dgeqrf", "zgeqrf", "dormqr", "dger", "dlange", "dorgqr", "dtpqrt",
           "dtpmqrt", "dtprfb", "dlarfb", "dlarft", "dlacpy", "dtrtri", "dgetri", "dsyevx", "dlatrd",
           "dsytrd", "dgemv", "dtrmm", "dpotrf", "dgetrs", "dgels", "dgesv"]


def reference_root():
    r = os.environ.get("CANDMC_REFERENCE", "/root/reference")
    return r if os.path.isfile(os.path.join(r, "alg", "QR", "qr_2d", "qr_2d.cxx")) else None


def openblas():
    import scipy
    d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
    c = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    if not c:
        raise RuntimeError("scipy's bundled OpenBLAS was not found")
    return os.path.abspath(c[0])


def _flags(ref):
    renames = [f"-D{f}_=scipy_{f}_" for f in FORTRAN]
    return ["-O3", "-fopenmp", "-fPIC", "-std=c++14", "-w", "-DFTN_UNDERSCORE=1", "-DLAPACKHASTSQR=1",
            "-I", os.path.join(HERE, "ref_shim"), "-I", ref, "-I", os.path.join(ref, "alg", "shared"),
            *renames]


def _compile(args):
    src, obj, flags = args
    r = subprocess.run(["g++", *flags, "-c", src, "-o", obj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on {src}:\n{r.stderr[-4000:]}")
    return obj


def build(force=False, verbose=False):
    ref = reference_root()
    if ref is None:
        if verbose:
            print("reference checkout not found: oracle/_ref not built")
        return None
    srcs = [os.path.join(ref, s) for s in SOURCES] + [os.path.join(HERE, "ref_shim", "ref_driver.cxx")]
    deps = srcs + [os.path.join(HERE, "ref_shim", "mpi.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    flags = _flags(ref)
    jobs = [(s, os.path.join(OUT, os.path.basename(s).replace(".cxx", ".o")), flags) for s in srcs]
    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as ex:
        objs = list(ex.map(_compile, jobs))
    blas = openblas()
    tmp = LIB + ".tmp"
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-o", tmp, *objs, blas,
                        f"-Wl,-rpath,{os.path.dirname(blas)}", "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
