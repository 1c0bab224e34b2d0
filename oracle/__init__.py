"""Oracle for the CANDMC QR hot path: a CPU restatement, the reference the tests check against.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py may import this package; the product library never
does and has no CPU fallback.

  lapack_restated  the LAPACK/BLAS routines the reference calls, restated
  candmc_oracle    bitree_tsqr / construct_Q1 / recursive_NLU / hh_recon_qr /
                   upd_A / QR_2D restated from the reference sources
  fixtures         the reference tests' srand48 fixture and the benchmark inputs

Parity anchor: the reference's arithmetic lives in LAPACK (>= 3.4.0).  The
restatement is pinned against LAPACK itself (scipy.linalg.lapack, run in the
tests) on the reference tests' own fixtures and pass criteria, and against
golden vectors committed in tests/golden/.
"""
