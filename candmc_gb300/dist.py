"""Sharded TSQR-HR and column-block trailing update across ranks.

The reference distributes a tall panel over a process column in b-row blocks
(bitree_tsqr.cxx:108-111), factors each block locally (local_tsqr, :155),
combines the b x b R factors up a binary tree whose pairs exchange packed
upper triangles (:172-232, b(b+1)/2 words per message), forms Q1 by walking
the tree back down (construct_tsqr_Q.cxx:147-217), runs the sign-choice LU on
the root (hh_recon.cxx:282), broadcasts W (:291) and forms Y2 = Q2 U^-1 on
every rank (:294-301).  The trailing update then needs Y and T on every
process column (the row broadcast of Y, qr_2d.cxx:168) and the Y^T A sums
over the process column (the column Allreduce, qr_2d.cxx:265).

On one GPU that whole grid is one device and none of this runs (the library
factors the panel with an on-chip tree).  This module is the multi-GPU form
of the same path for ranks that each own a GPU: the schedule, message
formats and collectives are the reference's, expressed with torch.distributed
point-to-point calls and broadcasts (NCCL between GPUs; gloo on CPU for the
tests), and the local arithmetic is delegated to a `kernels` object:

  local_qr(A)            -> (YR, tau)   Householder QR of the local block (dgeqrf form)
  tree_combine(R1, R2)   -> (R, V, tau) QR of [R1; R2], R2 upper (dtpqrt form)
  tree_apply(V, tau, C)  -> (top, bottom) Q_node [C; 0] (dtprfb, construct_tsqr_Q.cxx:195-208)
  leaf_apply(YR, tau, C) -> Q_leaf [C; 0]  (dormqr, construct_tsqr_Q.cxx:228-233)
  signed_lu(Q1top, R)    -> (LU, S R, signs) (hh_recon.cxx:43-110)
  trsm_upper(X, U)       -> X U^-1
  apply_qt(Y, T, C)      -> (I - Y T Y^T)^T C

`CudaKernels` binds them to this library's GPU entry points (bitree_tsqr,
tree_tsqr, recursive_NLU, upd_A); the b x b node products and the triangular
solve for Y2, which have no entry point of their own, are torch operations on
the rank's device.  Tensors are float64, column-major where they are matrices.
Every box of this build has a single GPU, so the multi-rank path runs in the
tests on CPU ranks (gloo) with the oracle as `kernels`; it is not measured on
GPUs.
"""
import torch


def tree_levels(np_work):
    """Levels of (receiver, sender) pairs, in ranks relative to the root, of
    the reference's binary tree (bitree_tsqr.cxx:172-232): at a level with np
    active ranks, relative rank r < np/2 receives from r + ceil(np/2)."""
    levels = []
    n = np_work
    while n > 1:
        levels.append([(r, r + (n + 1) // 2) for r in range(n // 2)])
        n = n // 2 + n % 2
    return levels


def pack_upper(R):
    """The reference's packed upper triangle (util.cxx:346-368): column by
    column, rows 0..j of column j; b(b+1)/2 values."""
    b = R.shape[1]
    return torch.cat([R[:j + 1, j] for j in range(b)])


def unpack_upper(p, b):
    R = torch.zeros((b, b), dtype=p.dtype, device=p.device)
    o = 0
    for j in range(b):
        R[:j + 1, j] = p[o:o + j + 1]
        o += j + 1
    return R


class ShardedPanel:
    """One rank's share of a panel factorization: its row block, leaf factor
    and the tree nodes it received at."""

    def __init__(self, A_local, b):
        self.A = A_local
        self.b = b
        self.nodes = []   # (level, sender, V, tau) for nodes this rank combined


def sharded_tsqr(A_local, b, kernels, group=None, root=0):
    """bitree_tsqr over the ranks of `group` (bitree_tsqr.cxx:91-248): every
    rank factors its block, then R factors are combined up the tree with
    packed-triangle messages.  Returns (panel, R): R (b x b) on the root, None
    elsewhere.  Every rank must hold at least b rows."""
    import torch.distributed as dist
    rank, p = dist.get_rank(group), dist.get_world_size(group)
    if A_local.shape[0] < b:
        raise ValueError("sharded_tsqr: every rank needs at least b rows")
    panel = ShardedPanel(A_local, b)
    panel.YR, panel.tau = kernels.local_qr(A_local)
    R = torch.triu(panel.YR[:b, :b])
    myr = (rank - root) % p
    for lvl, pairs in enumerate(tree_levels(p)):
        for recv, send in pairs:
            peer_recv, peer_send = (recv + root) % p, (send + root) % p
            if myr == send:
                dist.send(pack_upper(R).contiguous(), _global(peer_recv, group), group=group)
            elif myr == recv:
                buf = torch.empty(b * (b + 1) // 2, dtype=R.dtype, device=R.device)
                dist.recv(buf, _global(peer_send, group), group=group)
                R, V, tau = kernels.tree_combine(R, unpack_upper(buf, b))
                panel.nodes.append((lvl, peer_send, V, tau))
    return panel, (R if myr == 0 else None)


def sharded_construct_Q1(panel, kernels, group=None, root=0):
    """The first b columns of the tree Q, row block by row block
    (construct_tsqr_Q.cxx:147-233): the root starts from I, each receiver
    applies its node's reflectors to [C; 0] and sends the bottom b x b block
    to the sender, walking the levels in reverse; every rank then applies its
    leaf reflectors.  Returns this rank's Q1 rows."""
    import torch.distributed as dist
    rank, p = dist.get_rank(group), dist.get_world_size(group)
    b = panel.b
    myr = (rank - root) % p
    C = torch.eye(b, dtype=panel.YR.dtype, device=panel.YR.device) if myr == 0 else None
    levels = tree_levels(p)
    nodes = {lvl: (send, V, tau) for lvl, send, V, tau in panel.nodes}
    for lvl in range(len(levels) - 1, -1, -1):
        for recv, send in levels[lvl]:
            if myr == recv:
                peer, V, tau = nodes[lvl]
                C, bottom = kernels.tree_apply(V, tau, C)
                dist.send(bottom.contiguous(), _global(peer, group), group=group)
            elif myr == send:
                C = torch.empty((b, b), dtype=panel.YR.dtype, device=panel.YR.device)
                dist.recv(C, _global((recv + root) % p, group), group=group)
    return kernels.leaf_apply(panel.YR, panel.tau, C)


def sharded_hh_recon(A_local, b, kernels, group=None, root=0):
    """hh_recon_qr over the ranks of `group` (hh_recon.cxx:129-321): TSQR,
    Q1, the sign-choice LU of (Q1_top - S) on the root, W = U S broadcast to
    all, Y2 = Q2 U^-1 on every rank.  Returns (Y_local, R, W): this rank's rows
    of Y (the root's top b rows hold L, unit diagonal implicit, with S R above
    the diagonal, as in the reference's output buffer), R = S R and W."""
    import torch.distributed as dist
    rank, p = dist.get_rank(group), dist.get_world_size(group)
    myr = (rank - root) % p
    panel, R = sharded_tsqr(A_local, b, kernels, group, root)
    Q1 = sharded_construct_Q1(panel, kernels, group, root)
    W = torch.empty((b, b), dtype=Q1.dtype, device=Q1.device)
    signs = torch.empty(b, dtype=Q1.dtype, device=Q1.device)
    if myr == 0:
        LU, SR, s = kernels.signed_lu(Q1[:b].clone(), R)
        U = torch.triu(LU)
        W.copy_(U)
        signs.copy_(s)
    dist.broadcast(W, _global(root, group), group=group)     # hh_recon.cxx:291
    dist.broadcast(signs, _global(root, group), group=group)
    if myr == 0:
        Y = Q1.clone()
        if Y.shape[0] > b:
            Y[b:] = kernels.trsm_upper(Q1[b:], W)
        Y[:b] = torch.tril(LU, -1) + SR
        Rout = SR
    else:
        Y = kernels.trsm_upper(Q1, W)
        Rout = None
    return Y, Rout, W * signs[None, :]


def sharded_lstsq(A_local, b_local, kernels, group=None, root=0):
    """min ||A x - b|| for A (m x n) and b (m) split by rows over the ranks
    of `group`: the TSQR of [A | b] (n + 1 columns) up the reference's tree
    (sharded_tsqr) leaves R_aug = [[R, z], [0, rho]] on the root, with
    z = (Q^T b)[:n] and |rho| = ||b - A x||; the root solves R x = z and
    broadcasts x and |rho|.  Q is never formed.  Every rank needs at least
    n + 1 rows.  Returns (x, residual norm) on every rank."""
    import torch.distributed as dist
    rank, p = dist.get_rank(group), dist.get_world_size(group)
    myr = (rank - root) % p
    n = A_local.shape[1]
    Ab = torch.cat([A_local, b_local.reshape(-1, 1).to(A_local.dtype)], dim=1)
    _, R = sharded_tsqr(Ab, n + 1, kernels, group, root)
    out = torch.empty(n + 1, dtype=A_local.dtype, device=A_local.device)
    if myr == 0:
        x = torch.linalg.solve_triangular(R[:n, :n], R[:n, n:n + 1], upper=True)[:, 0]
        out[:n] = x
        out[n] = R[n, n].abs()
    dist.broadcast(out, _global(root, group), group=group)
    return out[:n].clone(), float(out[n])


def column_block_update(Y, T, A_cols, kernels, group=None, panel_rank=0):
    """update_A over a process row (qr_2d.cxx:124-177): the rank that factored
    the panel broadcasts Y (unit-lower, explicit) and T (hh_recon's output
    replicated, qr_2d.cxx:168,202); every rank applies (I - Y T Y^T)^T to the
    columns it owns.  Y and T are overwritten on the other ranks."""
    import torch.distributed as dist
    dist.broadcast(Y, _global(panel_rank, group), group=group)
    dist.broadcast(T, _global(panel_rank, group), group=group)
    return kernels.apply_qt(Y, T, A_cols)


def _global(r, group):
    import torch.distributed as dist
    return r if group is None else dist.get_global_rank(group, r)


class CudaKernels:
    """The local arithmetic on this rank's GPU through the library's C ABI."""

    def __init__(self):
        import candmc_gb300 as cm
        self.cm = cm
        cm.lib()

    def local_qr(self, A):
        A = self.cm.colmajor(A.clone())
        R, tau = self.cm.bitree_tsqr(A)
        return A, tau

    def tree_combine(self, R1, R2):
        b = R1.shape[0]
        S = self.cm.colmajor(torch.cat([R1, R2], 0))
        T = self.cm.tree_tsqr(S)
        V = torch.triu(S[b:])
        return torch.triu(S[:b]), V, torch.diagonal(self._full_T(V, T)).clone()

    def _full_T(self, V, Tblk):
        # the node's tau are the diagonal of the dtpqrt block factor
        b = V.shape[1]
        nb = Tblk.shape[0]
        T = torch.zeros((b, b), dtype=V.dtype, device=V.device)
        for c in range(b):
            T[c, c] = Tblk[c % nb, c]
        return T

    def tree_apply(self, V, tau, C):
        b = V.shape[1]
        Y = torch.cat([torch.eye(b, dtype=V.dtype, device=V.device), V], 0)
        X = self.cm.colmajor(torch.cat([C, torch.zeros_like(C)], 0))
        T = self._larft(Y, tau)
        X = X - Y @ (T @ (Y.t() @ X))
        return X[:b].clone(), X[b:].clone()

    def leaf_apply(self, YR, tau, C):
        m, b = YR.shape
        X = torch.zeros((m, C.shape[1]), dtype=C.dtype, device=C.device)
        X[:b] = C
        Y = torch.tril(YR, -1)
        Y[torch.arange(b), torch.arange(b)] = 1.0
        T = self._larft(Y, tau)
        return X - Y @ (T @ (Y.t() @ X))

    def _larft(self, Y, tau):
        b = Y.shape[1]
        G = Y.t() @ Y
        T = torch.zeros((b, b), dtype=Y.dtype, device=Y.device)
        for i in range(b):
            T[i, i] = tau[i]
            if i:
                T[:i, i] = -tau[i] * (T[:i, :i] @ G[:i, i])
        return T

    def signed_lu(self, Q1top, R):
        A = self.cm.colmajor(Q1top.clone())
        Rc = self.cm.colmajor(R.clone())
        s = self.cm.recursive_NLU(A, Rc)
        return A, Rc, s.to(A.dtype)

    def trsm_upper(self, X, U):
        return torch.linalg.solve_triangular(U, X, upper=True, left=False)

    def apply_qt(self, Y, T, C):
        # T from Y^T Y (upd_A with W = NULL, qr_2d.cxx:242-246): exact for the
        # reconstruction's reflectors, so the broadcast T is not needed here
        C = self.cm.colmajor(C)
        return self.cm.upd_A(self.cm.colmajor(Y), C, None)
