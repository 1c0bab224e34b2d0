"""CPU restatement of CANDMC's QR hot path: TSQR, Householder reconstruction, CAQR.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; the
tests, the smoke check and the CPU-baseline leg of the benchmark use it as
the reference result.

Each function restates one reference function (paths relative to the CANDMC
source tree) on numpy float64 arrays, with the LAPACK arithmetic from
`lapack_restated`.  The MPI process column of the reference is simulated in
one process: a "rank" is a contiguous block of rows, the binary tree pairs
ranks exactly as alg/QR/tsqr/bitree_tsqr.cxx:172-232 does, and the messages
become array hand-offs.  With numPes == 1 every function reduces to the
reference's single-rank path, which is the one a single GPU replaces.
"""
import numpy as np

from . import lapack_restated as lp

BSIZE = 64      # recursion base of recursive_NLU, alg/QR/hh_recon/hh_recon.cxx:13


# --------------------------------------------------------------------------
# row distribution (alg/QR/hh_recon/hh_recon.cxx:144-145, bitree_tsqr.cxx:110-111)
# --------------------------------------------------------------------------
def local_rows(m, b, numPes, myRank, root=0):
    """Rows owned by myRank: ((m/b)/numPes)*b, plus b for the first (m/b)%numPes ranks after root."""
    mb = ((m // b) // numPes) * b
    if (m // b) % numPes > (myRank + numPes - root) % numPes:
        mb += b
    return mb


def split_rows(A, b, numPes, root=0):
    """Contiguous row blocks per rank, ranks ordered root, root+1, ... (the test layout)."""
    m = A.shape[0]
    sizes = [local_rows(m, b, numPes, r, root) for r in range(numPes)]
    order = [(root + i) % numPes for i in range(numPes)]
    blocks, off = {}, 0
    for r in order:
        blocks[r] = A[off:off + sizes[r], :].copy()
        off += sizes[r]
    assert off == m, "m must be a multiple of b for the multi-rank layout"
    return [blocks[r] for r in range(numPes)], order


def join_rows(blocks, order):
    return np.vstack([blocks[r] for r in order])


# --------------------------------------------------------------------------
# TSQR (alg/QR/tsqr/bitree_tsqr.cxx)
# --------------------------------------------------------------------------
def local_tsqr(A):
    """Leaf QR by dgeqrf (bitree_tsqr.cxx:48-71).  A becomes Y\\R, returns tau."""
    return lp.dgeqrf(A)


def tree_tsqr(R1, R2):
    """Tree-node QR of [R1; R2] by dtpqrt (bitree_tsqr.cxx:20-34).

    R1 (top, upper) becomes R; R2 (bottom, upper) becomes the reflector block V.
    Returns tau of the node reflectors.
    """
    return lp.dtpqrt_tri(R1, R2)


def tree_schedule(np_work):
    """Binary-tree pairing of bitree_tsqr.cxx:172-232: list of levels of (receiver, sender) relative ranks."""
    levels = []
    np_ = np_work
    while np_ > 1:
        pairs = []
        for myr in range(np_ // 2):
            pairs.append((myr, myr + (np_ + 1) // 2))
        levels.append(pairs)
        np_ = np_ // 2 + np_ % 2
    return levels


def bitree_tsqr(blocks, b, root=0):
    """Binary-tree TSQR over a simulated process column (bitree_tsqr.cxx:91-248).

    blocks[r] (mb_r x b) is rank r's piece; it is overwritten with the leaf
    Y\\R (output_Y = 1).  Returns (R, taus, tree): R (b x b, zero below the
    diagonal) at the root, taus[r] the leaf tau of rank r, tree the list of
    levels, each a list of (receiver_rank, sender_rank, V, tau).
    """
    numPes = len(blocks)
    m = sum(blk.shape[0] for blk in blocks)
    np_work = m // b if numPes * b > m else numPes
    taus = [local_tsqr(blk) for blk in blocks]
    if np_work == 1:
        R = np.triu(blocks[root][:b, :b])
        return R, taus, []
    Rs = {r: np.triu(blocks[r][:b, :b]).copy() for r in range(numPes)}
    tree = []
    for pairs in tree_schedule(np_work):
        level = []
        for myr_recv, myr_send in pairs:
            rr = (myr_recv + root) % numPes
            rs = (myr_send + root) % numPes
            R1, R2 = Rs[rr], Rs[rs].copy()
            tau = tree_tsqr(R1, R2)
            level.append((rr, rs, np.triu(R2), tau))
        tree.append(level)
    return np.triu(Rs[root]), taus, tree


def construct_Q1(blocks_Y, taus, tree, b, k, root=0):
    """Explicit first k columns of the TSQR Q (construct_tsqr_Q.cxx:34-242).

    Tree descent applies each node's reflectors to [C_receiver; 0]
    (dtprfb, :195-208); each leaf then applies its own reflectors to
    [C_r; 0] (dormqr, :228-233).  For one rank this is dorgqr (:96).
    Returns the list of per-rank Q1 blocks.
    """
    numPes = len(blocks_Y)
    if not tree:
        out = []
        for r in range(numPes):
            mb = blocks_Y[r].shape[0]
            Q = np.zeros((mb, k))
            if r == root:
                Q[:, :] = blocks_Y[r][:, :k]
                lp.dorg2r(Q, taus[r][:b] if k >= b else taus[r][:k], ncols=k)
            out.append(Q)
        return out
    C = {r: np.zeros((b, k)) for r in range(numPes)}
    C[root][:min(b, k), :min(b, k)] = np.eye(min(b, k))
    for level in reversed(tree):
        for rr, rs, V, tau in level:
            top, bottom = C[rr], np.zeros((b, k))
            lp.dtpmqrt_left_notrans(V, tau, top, bottom)
            C[rs] = bottom
    out = []
    for r in range(numPes):
        Yr = blocks_Y[r]
        mb = Yr.shape[0]
        Q = np.zeros((mb, k))
        Q[:b, :] = C[r]
        lp.dormqr_left_notrans(Yr, taus[r], Q)
        out.append(Q)
    return out


def apply_tsqr_QT(YR, tau, B, b):
    """B <- Q^T B for the single-rank TSQR factor (apply_tsqr_QT.cxx:74-82:
    dormqr('L','T') with the leaf's reflectors): B - Y T^T (Y^T B), T from
    dlarft.  YR holds the dgeqrf-form reflectors below its diagonal."""
    Y = lp.unit_lower(YR, b)
    T = lp.dlarft(Y, tau)
    return B - Y @ (T.T @ (Y.T @ B))


# --------------------------------------------------------------------------
# Householder reconstruction (alg/QR/hh_recon/hh_recon.cxx)
# --------------------------------------------------------------------------
def signed_NLU(A, R, signs, off=0):
    """Sign-choice unpivoted LU of (A - S) in place (hh_recon.cxx:43-68).

    S_ii = -sign(A_ii) (+1 when A_ii <= 0); rows of R with S_ii = -1 are
    negated from the diagonal on.  A becomes L\\U.  signs[off:off+b] filled.
    """
    b = A.shape[0]
    for i in range(b):
        s = -1 if A[i, i] > 0 else 1
        signs[off + i] = s
        A[i, i] -= s
        if s == -1:
            R[i, i:] *= -1.0
        A[i + 1:, i] /= A[i, i]
        A[i + 1:, i + 1:] -= np.outer(A[i + 1:, i], A[i, i + 1:])


def recursive_NLU(A, R, signs=None, off=0):
    """Recursive signed LU, halving until b <= BSIZE (hh_recon.cxx:80-110)."""
    b = A.shape[0]
    if signs is None:
        signs = np.zeros(b, dtype=np.int64)
    if b <= BSIZE:
        signed_NLU(A, R, signs, off)
        return signs
    b1 = b // 2
    recursive_NLU(A[:b1, :b1], R[:b1, :b1], signs, off)
    for i in range(b1):
        if signs[off + i] == -1:
            R[i, b1:] *= -1.0
    lp.dtrsm('L', 'L', 'N', 'U', 1.0, A[:b1, :b1], A[:b1, b1:])
    lp.dtrsm('R', 'U', 'N', 'N', 1.0, A[:b1, :b1], A[b1:, :b1])
    A[b1:, b1:] -= A[b1:, :b1] @ A[:b1, b1:]
    recursive_NLU(A[b1:, b1:], R[b1:, b1:], signs, off + b1)
    return signs


def hh_recon_qr(A, b, numPes=1, root=0):
    """TSQR + Householder reconstruction of an m x b panel (hh_recon.cxx:129-321).

    Returns (YR, W): YR (m x b) holds Y (strictly lower, unit diagonal
    implicit) and S*R (upper); W (b x b, upper) = U*S = -T*Y1^T.  A is not
    modified.  numPes > 1 runs the binary tree over that many simulated ranks.
    """
    A = np.array(A, dtype=np.float64)
    m = A.shape[0]
    assert A.shape[1] == b
    if numPes == 1:
        blocks, order = [A], [0]
    else:
        blocks, order = split_rows(A, b, numPes, root)
    R, taus, tree = bitree_tsqr(blocks, b, root)
    Q1s = construct_Q1(blocks, taus, tree, b, b, root)
    Q1r = Q1s[root]
    Rw = R.copy()
    signs = recursive_NLU(Q1r[:b, :b], Rw)
    U = np.triu(Q1r[:b, :b])
    W = U.copy()
    for r in range(numPes):
        Q1 = Q1s[r]
        if r == root:
            lp.dtrsm('R', 'U', 'N', 'N', 1.0, U, Q1[b:, :])
            Yblk = np.tril(Q1, -1)
            Yblk[:b, :] += np.triu(Rw)
            blocks[r] = Yblk
        else:
            lp.dtrsm('R', 'U', 'N', 'N', 1.0, U, Q1)
            blocks[r] = Q1
    for i in range(b):
        if signs[i] == -1:
            W[:i + 1, i] *= -1.0
    YR = join_rows(blocks, order) if numPes > 1 else blocks[0]
    return YR, W


def compute_invT_from_W(W, Y1):
    """T^-T from W and the unit-lower top block Y1: solve W^T X = -Y1 (hh_recon.cxx:26-31)."""
    X = np.array(Y1, dtype=np.float64)
    lp.dtrsm('L', 'U', 'T', 'N', -1.0, W, X)
    return np.tril(X)


def compute_invT_from_Y(Y):
    """T^-T = stril(Y^T Y) with halved diagonal (qr_2d.cxx:22-60)."""
    G = Y.T @ Y
    X = np.tril(G, -1)
    X[np.diag_indices_from(X)] = np.diag(G) / 2.0
    return X


def compute_invT_from_Y2(Y1, Y2):
    """Rectangular Y1^T Y2 (qr_2d.cxx:76-106)."""
    return Y1.T @ Y2


def T_from_W(W, Y1):
    """Upper-triangular T with W = -T*Y1^T, i.e. T = (T^-T)^-T."""
    X = compute_invT_from_W(W, Y1)
    return np.linalg.inv(X).T


def upd_A(Y, A, W=None, W_is_T=False):
    """Trailing update A <- (I - Y T Y^T)^T A = A - Y T^T (Y^T A)  (qr_2d.cxx:224-282).

    Y: explicit unit-lower-trapezoidal m x b.  W: None (T^-T from Y^T Y),
    W = -T*Y1^T (the hh_recon_qr output), or, with W_is_T, the lower T^-T
    itself.  Z = Y^T A (dgemm :259), Z <- (T^-T)^-1 Z (dtrsm :271),
    A -= Y Z (dgemm :275).  A is updated in place and returned.
    """
    b = Y.shape[1]
    if W is None:
        X = compute_invT_from_Y(Y)
    elif W_is_T:
        X = np.tril(W)
    else:
        X = compute_invT_from_W(W, Y[:b, :b])
    Z = Y.T @ A
    lp.dtrsm('L', 'L', 'N', 'N', 1.0, X, Z)
    A -= Y @ Z
    return A


def update_A(YR, A, b, W):
    """update_A on one rank (qr_2d.cxx:124-177): Y packed with unit diagonal, then upd_A."""
    Y = lp.unit_lower(YR, b)
    return upd_A(Y, A, W)


def QR_2D(A, b):
    """Right-looking CAQR on a 1 x 1 process grid (qr_2d.cxx:299-363).

    Each panel: hh_recon_qr on the first min(k,b) columns (:313), then
    update_A of the trailing columns (:325), then recurse on the trailing
    (m-b) x (k-b) block (:339).  A (m x k) is overwritten with Y\\R.
    Returns the list of per-panel W.
    """
    A = np.asarray(A)
    m, k = A.shape
    Ws = []
    r0 = 0
    while True:
        mm, kk = m - r0, k - r0
        bb = min(kk, b)
        YR, W = hh_recon_qr(A[r0:, r0:r0 + bb], bb)
        A[r0:, r0:r0 + bb] = YR
        Ws.append(W)
        if kk - b > 0 and mm - b > 0:
            update_A(A[r0:, r0:r0 + b], A[r0:, r0 + b:], b, W)
            r0 += b
        else:
            break
    return Ws


def ls_solve(A, B, b):
    """Least-squares oracle: QR_2D on the augmented [A | B] (the right-hand
    sides receive Q^T B through the reference's own update_A), then
    X = R^-1 (Q^T B)[0:n] by back substitution (dtrsm)."""
    m, n = A.shape
    Aug = np.hstack([np.asarray(A, dtype=np.float64), np.asarray(B, dtype=np.float64)])
    # factor only the first n columns: panels never start inside B
    r0 = 0
    while r0 < n:
        bb = min(b, n - r0)
        YR, W = hh_recon_qr(Aug[r0:, r0:r0 + bb], bb)
        Aug[r0:, r0:r0 + bb] = YR
        # every panel's Q^T reaches B, including a square last panel (whose
        # reconstructed last reflector is a sign flip, not the identity)
        update_A(Aug[r0:, r0:r0 + bb], Aug[r0:, r0 + bb:], bb, W)
        r0 += bb
    R = np.triu(Aug[:n, :n])
    X = np.array(Aug[:n, n:])
    lp.dtrsm('L', 'U', 'N', 'N', 1.0, R, X)
    return X


def tau_recon(structure, Y, nrow=None):
    """tau_recon (alg/shared/util.cxx:437-466): tau_i = 2/(1 + ||y_i||^2) over
    column i's part -- 'R' rows 0..nrow-1, 'L' rows i+1..nrow-1, 'U' rows
    0..i -- mapped to 0 where it equals 2."""
    Y = np.asarray(Y)
    nrow = Y.shape[0] if nrow is None else nrow
    tau = np.zeros(Y.shape[1])
    for i in range(Y.shape[1]):
        lo, hi = {"R": (0, nrow), "L": (i + 1, nrow), "U": (0, i + 1)}[structure]
        nrm = np.linalg.norm(Y[lo:hi, i])
        t = 2.0 / (nrm * nrm + 1.0)
        tau[i] = 0.0 if t == 2.0 else t
    return tau


def tau_recon_lower(Y, b, lapack_zero=False):
    """tau_i = 2/(1 + ||Y[i+1:, i]||^2) (alg/shared/util.cxx:437-466, 'L').

    The reference maps tau = 2 (an empty reflector tail) to 0, LAPACK's
    choice for that case (lapack_zero=True).  Reconstruction keeps tau = 2
    there: its sign choice S makes the reflector a sign flip, which is how
    the last column of a square panel gets R_bb's sign (the reference's
    test_qr_2d.cxx:135-138 notes the resulting difference from LAPACK).  The
    checks below use the reconstruction convention.
    """
    tau = np.zeros(b)
    for i in range(b):
        nrm = np.linalg.norm(Y[i + 1:, i])
        t = 2.0 / (nrm * nrm + 1.0)
        tau[i] = 0.0 if (lapack_zero and t == 2.0) else t
    return tau


# --------------------------------------------------------------------------
# checks used by the reference tests
# --------------------------------------------------------------------------
def q_from_yr(YR, b, ncols=None):
    """Explicit Q (m x ncols) of the Householder factor stored in YR (tau from tau_recon)."""
    m = YR.shape[0]
    Y = lp.unit_lower(YR, b)
    tau = tau_recon_lower(YR, b)
    T = lp.dlarft(Y, tau)
    n = b if ncols is None else ncols
    E = np.zeros((m, n))
    E[:n, :n] = np.eye(n)
    return E - Y @ (T @ (Y[:n, :].T))


def column_relative_residual(A, YR, b):
    """sum_j ||(A - QR) e_j|| / ||A e_j||, the pass metric of test/QR/test_hh_recon.cxx:236-259."""
    m = A.shape[0]
    tau = tau_recon_lower(YR, b)
    R = np.zeros((m, b))
    R[:b, :] = np.triu(YR[:b, :b])
    QR = lp.dormqr_left_notrans(YR, tau, R)
    D = A - QR
    return float(sum(np.linalg.norm(D[:, j]) / np.linalg.norm(A[:, j]) for j in range(b)))


def backward_error(A, YR, ks=None):
    """||A - QR||_F / ||A||_F for a full CAQR output YR of A (m x k)."""
    m, k = A.shape
    kk = min(m, k)
    Y = lp.unit_lower(YR, kk)
    tau = tau_recon_lower(YR, kk)
    R = np.triu(YR[:kk, :])
    Rf = np.zeros((m, k))
    Rf[:kk, :] = R
    QR = lp.dormqr_left_notrans(YR, tau, Rf)
    return float(np.linalg.norm(A - QR) / np.linalg.norm(A))


def orthogonality_error(YR, b):
    """||I - Q^T Q||_F of the first b columns of the Householder Q in YR."""
    Q = q_from_yr(YR, b)
    return float(np.linalg.norm(np.eye(b) - Q.T @ Q))
