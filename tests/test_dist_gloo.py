"""The sharded (multi-rank) TSQR-HR and column-block update of
candmc_gb300/dist.py on CPU ranks over gloo, with the oracle as the local
arithmetic.

Checks, for 2 and 3 ranks and a rotated root:
* the tree schedule is the reference's (bitree_tsqr.cxx:172-232, restated in
  the oracle's tree_schedule);
* the sharded hh_recon gives the canonical (Y, S*R, W) of the single-rank
  factorization of the whole panel (the reconstruction's output does not
  depend on the process count, hh_recon.cxx:129-321) -- within 1e-12;
* the column-block update, with Y and T broadcast from the panel's rank,
  equals upd_A on the whole matrix (qr_2d.cxx:124-177) -- within 1e-12;
* the sharded least-squares solve (the TSQR of [A | b] up the same tree)
  matches LAPACK's lstsq on the whole system -- within 1e-12, with the
  residual norm.
The ranks are separate processes (spawned) talking to each other only through
torch.distributed on 127.0.0.1.  Not measured on GPUs: every box of this
build has one GPU.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from candmc_gb300 import dist as cdist  # noqa: E402
from oracle import candmc_oracle as co  # noqa: E402
from oracle import fixtures as fx  # noqa: E402
from oracle import lapack_restated as lp  # noqa: E402


class OracleKernels:
    """The dist module's local arithmetic, on numpy through the oracle."""

    @staticmethod
    def _t(x):
        return torch.from_numpy(np.ascontiguousarray(x))

    def local_qr(self, A):
        YR = np.array(A.numpy(), order="F")
        tau = lp.dgeqrf(YR)
        return self._t(YR), self._t(tau)

    def tree_combine(self, R1, R2):
        r1, r2 = np.array(R1.numpy()), np.array(R2.numpy())
        tau = lp.dtpqrt_tri(r1, r2)
        return self._t(np.triu(r1)), self._t(np.triu(r2)), self._t(tau)

    def tree_apply(self, V, tau, C):
        top, bottom = np.array(C.numpy()), np.zeros_like(C.numpy())
        lp.dtpmqrt_left_notrans(V.numpy(), tau.numpy(), top, bottom)
        return self._t(top), self._t(bottom)

    def leaf_apply(self, YR, tau, C):
        Q = np.zeros((YR.shape[0], C.shape[1]))
        Q[:C.shape[0]] = C.numpy()
        lp.dormqr_left_notrans(YR.numpy(), tau.numpy(), Q)
        return self._t(Q)

    def signed_lu(self, Q1top, R):
        A, Rr = np.array(Q1top.numpy()), np.array(R.numpy())
        s = co.recursive_NLU(A, Rr)
        return self._t(A), self._t(Rr), self._t(np.asarray(s, dtype=np.float64))

    def trsm_upper(self, X, U):
        import scipy.linalg as sl
        return self._t(sl.solve_triangular(U.numpy(), X.numpy().T, trans="T", lower=False).T)

    def apply_qt(self, Y, T, C):
        return self._t(co.upd_A(Y.numpy(), np.array(C.numpy()), None))


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, m, b, root, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        A = fx.gaussian(m, b, 5 * m + b)
        rows = np.array_split(np.arange(m), world)
        # relative rank r of the tree owns row block r (the reference's cyclic rotation by root)
        myr = (rank - root) % world
        blk = torch.from_numpy(np.ascontiguousarray(A[rows[myr]]))
        Y, R, W = cdist.sharded_hh_recon(blk, b, OracleKernels(), root=root)
        # column-block update of a trailing matrix split by columns over the ranks
        C = fx.gaussian(m, 2 * world + 3, 7)
        cols = np.array_split(np.arange(C.shape[1]), world)[rank]
        Yfull = torch.zeros((m, b), dtype=torch.float64)
        Ttmp = torch.zeros((b, b), dtype=torch.float64)
        nmax = max(len(r) for r in rows)
        parts = [torch.zeros((nmax, b), dtype=torch.float64) for _ in range(world)]
        dist.all_gather(parts, _pad(Y, nmax))
        for r_rel in range(world):
            Yfull[rows[r_rel]] = parts[(r_rel + root) % world][:len(rows[r_rel])]
        Yu = torch.tril(Yfull, -1)
        Yu[torch.arange(b), torch.arange(b)] = 1.0
        newC = cdist.column_block_update(Yu.clone() if rank == root else torch.zeros_like(Yu), Ttmp,
                                         torch.from_numpy(np.ascontiguousarray(C[:, cols])), OracleKernels(),
                                         panel_rank=root)
        out[rank] = {"Y": Yfull.numpy(), "R": None if R is None else R.numpy(), "W": W.numpy(),
                     "C": newC.numpy(), "cols": cols}
    finally:
        dist.destroy_process_group()


def _pad(Y, n):
    P = torch.zeros((n, Y.shape[1]), dtype=Y.dtype)
    P[:Y.shape[0]] = Y
    return P


def _run(world, m, b, root):
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = _port()
    mp.start_processes(_worker, args=(world, port, m, b, root, out), nprocs=world, join=True,
                       start_method="spawn")
    return dict(out)


def test_tree_levels_are_the_reference_schedule():
    for p in range(1, 10):
        assert [list(l) for l in cdist.tree_levels(p)] == [list(l) for l in co.tree_schedule(p)]


def test_packed_triangle_round_trip():
    R = torch.triu(torch.arange(1.0, 26.0, dtype=torch.float64).reshape(5, 5))
    p = cdist.pack_upper(R)
    assert p.numel() == 15 and p[:3].tolist() == [1.0, 2.0, 7.0]
    assert torch.equal(cdist.unpack_upper(p, 5), R)


@pytest.mark.parametrize("world,m,b,root", [(2, 96, 16, 0), (3, 150, 12, 1), (2, 64, 32, 1), (3, 100, 16, 2)])
def test_sharded_hh_recon_and_update(world, m, b, root):
    out = _run(world, m, b, root)
    A = fx.gaussian(m, b, 5 * m + b)
    YR1, W1 = co.hh_recon_qr(A, b)                      # single rank, canonical
    Y = out[root]["Y"]
    scale = max(1.0, np.abs(YR1).max())
    assert np.abs(np.tril(Y, -1) - np.tril(YR1, -1)).max() <= 1e-12 * scale
    assert np.abs(out[root]["R"] - np.triu(YR1[:b])).max() <= 1e-12 * scale
    for r in range(world):
        assert np.abs(np.triu(out[r]["W"]) - np.triu(W1)).max() <= 1e-12
    # the column blocks, against upd_A on the whole trailing matrix
    C = fx.gaussian(m, 2 * world + 3, 7)
    Yu = lp.unit_lower(YR1, b)
    want = co.upd_A(Yu, C.copy(), None)
    for r in range(world):
        cols = out[r]["cols"]
        assert np.abs(out[r]["C"] - want[:, cols]).max() <= 1e-12 * max(1.0, np.abs(want).max())


def _ls_worker(rank, world, port, m, n, root, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        A = fx.gaussian(m, n, 11 * m + n)
        bvec = fx.gaussian(m, 1, 13 * m + n)[:, 0]
        rows = np.array_split(np.arange(m), world)
        myr = (rank - root) % world
        x, rho = cdist.sharded_lstsq(torch.from_numpy(np.ascontiguousarray(A[rows[myr]])),
                                     torch.from_numpy(np.ascontiguousarray(bvec[rows[myr]])),
                                     OracleKernels(), root=root)
        out[rank] = {"x": x.numpy(), "rho": rho}
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,m,n,root", [(2, 300, 12, 0), (3, 400, 20, 1)])
def test_sharded_lstsq(world, m, n, root):
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_ls_worker, args=(world, _port(), m, n, root, out), nprocs=world, join=True,
                       start_method="spawn")
    A = fx.gaussian(m, n, 11 * m + n)
    bvec = fx.gaussian(m, 1, 13 * m + n)[:, 0]
    xo, res, _, _ = np.linalg.lstsq(A, bvec, rcond=None)
    for r in range(world):
        x = out[r]["x"]
        assert np.linalg.norm(x - xo) <= 1e-12 * np.linalg.norm(xo)
        assert abs(out[r]["rho"] - np.linalg.norm(bvec - A @ xo)) <= 1e-12 * np.linalg.norm(bvec)
