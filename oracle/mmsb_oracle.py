"""FP64 CPU restatement of the reference's MMSB tensor-method path -- the ORACLE.

This module is test infrastructure: only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use it, always as the oracle results are compared
with, never as the thing measured or shipped.  The GPU library never calls it.

Parity is pinned by tests/golden/: fixtures produced by the reference's own CPU
implementation (CommunityDetectionSoftware_CPU, compiled unmodified by
oracle/Makefile with a fixed srand seed, see oracle/ref_harness.cpp) on seeded
synthetic graphs.  tests/test_oracle_golden.py checks every stage of this file
against them.

Each function cites the reference code it restates (paths relative to
CommunityDetectionSoftware_CPU/CommunityDetection/ unless noted).  The
reference forms the n x n pair operators explicitly (Util.cpp:54-62); here they
are applied implicitly as chains of sparse products, which is the same algebra
in a different association order.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

TOLERANCE = 1e-6  # stdafx.h:59


def pinv_vector(v, tol=TOLERANCE):
    """Spectral.cpp:50-57: elementwise 1/x, 0 where |x| <= tol."""
    v = np.asarray(v, dtype=np.float64)
    out = np.zeros_like(v)
    m = np.abs(v) > tol
    out[m] = 1.0 / v[m]
    return out


def orthogonalize_cols(Y, tol=TOLERANCE):
    """Spectral.cpp:146-166: modified Gram-Schmidt, columns with norm <= tol -> 0."""
    Y = np.array(Y, dtype=np.float64, copy=True)
    c = Y.shape[1]
    for j in range(c):
        for i in range(j):
            Y[:, j] -= (Y[:, i] @ Y[:, j]) * Y[:, i]
        nrm = np.sqrt(Y[:, j] @ Y[:, j])
        Y[:, j] *= (1.0 / nrm) if nrm > tol else 0.0
    return Y


def orthogonalize_cols_cgs2(Y, tol=TOLERANCE, block=32):
    """The same column orthonormalisation with classical Gram-Schmidt applied
    twice per column, blocked (each block of columns is projected against the
    finished ones twice with matrix products, then orthonormalised column by
    column with the same drop rule); equal to orthogonalize_cols to round-off.
    Used where the oracle is timed on large inputs.  When every column keeps
    a residual well above tol (the Householder R's diagonal shows it), no
    column is dropped and the result is the Q of the QR factorisation with a
    positive R diagonal, which Householder QR gives directly."""
    Y = np.array(Y, dtype=np.float64, copy=True)
    n, c = Y.shape
    if n >= c:
        Qh, R = np.linalg.qr(Y)
        d = np.abs(np.diag(R))
        if d.min() > 2.0 * tol:
            return Qh * np.where(np.diag(R) < 0, -1.0, 1.0)
    Q = np.zeros_like(Y)
    for j0 in range(0, c, block):
        j1 = min(c, j0 + block)
        V = Y[:, j0:j1].copy()
        for _ in range(2):
            if j0:
                V -= Q[:, :j0] @ (Q[:, :j0].T @ V)
        for j in range(j0, j1):
            v = V[:, j - j0]
            for _ in range(2):
                if j > j0:
                    v -= Q[:, j0:j] @ (Q[:, j0:j].T @ v)
            nrm = np.sqrt(v @ v)
            Q[:, j] = v * ((1.0 / nrm) if nrm > tol else 0.0)
    return Q


FAST_GS = False  # True: orthogonalize_cols_cgs2 inside svd_sym_nystrom
SPMM_THREADS = 1  # > 1: sparse x dense products split by rows over host threads


def _mm(A, P):
    """A @ P; with SPMM_THREADS > 1 and a sparse A, row blocks of the product
    run on a thread pool (scipy's sparse kernels release the GIL; every row is
    computed exactly as in the single product)."""
    if SPMM_THREADS <= 1 or not sp.issparse(A) or A.shape[0] < 4096 or np.ndim(P) != 2:
        return A @ P
    from concurrent.futures import ThreadPoolExecutor
    A = A.tocsr()
    nt = SPMM_THREADS
    bounds = np.linspace(0, A.shape[0], nt + 1).astype(np.int64)
    out = np.empty((A.shape[0], P.shape[1]), dtype=np.result_type(A.dtype, P.dtype))

    def run(i):
        out[bounds[i]:bounds[i + 1]] = A[bounds[i]:bounds[i + 1]] @ P

    with ThreadPoolExecutor(nt) as ex:
        list(ex.map(run, range(nt)))
    return out


def svd_sym_nystrom(M, k, rows_factor=20, tol=TOLERANCE):
    """Spectral.cpp:169-223 (SVD_symNystrom_sparse) for an n x 2k input.

    Returns (U: n x k, sigma: k).  Nystrom branch when rows > rows_factor*k:
    Q = orth(M); C = M * Q[:cols]; Z = C^T C; U = C V_k S_k^{-1/2}, sigma = sqrt(S_k).
    Otherwise the thin SVD of M (Spectral.cpp:216-221)."""
    M = np.asarray(M, dtype=np.float64)
    n, cols = M.shape
    if n > rows_factor * k:
        if cols > 2 * k:
            raise NotImplementedError("sketching branch (Spectral.cpp:176-178) is unused here")
        Q = (orthogonalize_cols_cgs2 if FAST_GS else orthogonalize_cols)(M, tol)
        QQ = Q[:cols, :] if cols < Q.shape[0] else Q
        C = M @ QQ
        Z = C.T @ C
        evals, evecs = np.linalg.eigh(Z)
        order = np.argsort(evals)[::-1]
        S = np.maximum(evals[order][:k], 0.0)
        V = evecs[:, order][:, :k]
        sigma = np.sqrt(S)
        U = (C @ V) * pinv_vector(np.sqrt(S), tol)
        return U, sigma
    U, s, _ = np.linalg.svd(M, full_matrices=False)
    return U[:, :k], s[:k]


def pinv_component(X, XT, R, k, rows_factor=20, tol=TOLERANCE):
    """Spectral.cpp:296-315 via SVD_asymNystrom_sparse (:225-246).

    X / XT apply the (implicit) matrix and its transpose to a dense panel.
    Returns (V: cols x k, U: rows x k, L_inv: k) with pinv(X) ~ V diag(L_inv) U^T."""
    gram = XT(X(R))                        # X^T (X R)
    V, s = svd_sym_nystrom(gram, k, rows_factor, tol)
    Linv_sqrt = np.sqrt(pinv_vector(s, tol))
    U = X(V) * Linv_sqrt                   # X V L^{-1/2}
    L = np.sqrt(s)
    return V, U, pinv_vector(L, tol)


def column_means(G, inv):
    return inv * np.asarray(G.sum(axis=0)).ravel()


def second_whiten(Gxa, Gxb, Gxc, k, alpha0, sketches, rows_factor=20, normalize=True,
                  tol=TOLERANCE):
    """Util.cpp:38-127.  sketches = (R_c: n_B x 2k, R_b: n_C x 2k, R_a: n_A x 2k).

    Returns dict W, Zb1, Zb2, Zc1, Zc2, mu_a, mu_b, mu_c (+ intermediates)."""
    nx = Gxa.shape[0]
    inv = 1.0 / nx if normalize else 1.0
    mu_a, mu_b, mu_c = column_means(Gxa, inv), column_means(Gxb, inv), column_means(Gxc, inv)
    Gxa, Gxb, Gxc = (sp.csr_matrix(g, dtype=np.float64) for g in (Gxa, Gxb, Gxc))
    GaT, GbT, GcT = Gxa.T.tocsr(), Gxb.T.tocsr(), Gxc.T.tocsr()
    zb_num = lambda P: inv * _mm(GaT, _mm(Gxc, P))    # Gx_a^T Gx_c (n_A x n_C)
    zb_den = lambda P: inv * _mm(GbT, _mm(Gxc, P))    # Gx_b^T Gx_c (n_B x n_C)
    zb_den_T = lambda P: inv * _mm(GcT, _mm(Gxb, P))
    zc_num = lambda P: inv * _mm(GaT, _mm(Gxb, P))    # Gx_a^T Gx_b (n_A x n_B)
    zc_den = lambda P: inv * _mm(GcT, _mm(Gxb, P))    # Gx_c^T Gx_b (n_C x n_B)
    zc_den_T = lambda P: inv * _mm(GbT, _mm(Gxc, P))
    R_c, R_b, R_a = (np.asarray(r, dtype=np.float64) for r in sketches)

    V_c, U_c, Linv_c = pinv_component(zc_den, zc_den_T, R_c, k, rows_factor, tol)
    V_b, U_b, Linv_b = pinv_component(zb_den, zb_den_T, R_b, k, rows_factor, tol)
    Zc1 = zc_num(V_c) * Linv_c                     # term_na_k  (Util.cpp:83-84)
    Zc2 = U_c.T                                    # (Util.cpp:85)
    core = U_c.T @ zc_den(U_b)                     # term_k_k   (Util.cpp:90)
    if np.count_nonzero(core) < k:                 # (Util.cpp:91-94)
        core[np.arange(k), np.arange(k)] = 1.0
    Zb1 = zb_num(V_b) * Linv_b                     # term_k_na^T (Util.cpp:96-97)
    Zb2 = U_b.T                                    # (Util.cpp:98)
    M2 = (alpha0 + 1.0) * ((Zc1 @ core) @ (Zb1.T @ R_a))      # (Util.cpp:103-104)
    M2 -= alpha0 * np.outer(mu_a, mu_a @ R_a)                  # (Util.cpp:110-112)
    Uw, sw = svd_sym_nystrom(M2, k, rows_factor, tol)          # (Util.cpp:116)
    W = Uw * pinv_vector(np.sqrt(sw), tol)                     # (Util.cpp:118-123)
    return dict(W=W, Zb1=Zb1, Zb2=Zb2, Zc1=Zc1, Zc2=Zc2, mu_a=mu_a, mu_b=mu_b, mu_c=mu_c,
                core=core, M2=M2, sw=sw, V_c=V_c, U_c=U_c, V_b=V_b, U_b=U_b,
                Linv_c=Linv_c, Linv_b=Linv_b)


def whitened_data(Gxa, Gxb, Gxc, wh):
    """CommunityDetection.cpp:66-68: Data_P = (effective W_P)^T G_XP^T, k x n_X."""
    W = wh["W"]
    Wb = wh["Zb2"].T @ (wh["Zb1"].T @ W)           # ((W^T Zb1) Zb2)^T
    Wc = wh["Zc2"].T @ (wh["Zc1"].T @ W)
    Da = np.asarray(_mm(Gxa, W).T)
    Db = np.asarray(_mm(Gxb, Wb).T)
    Dc = np.asarray(_mm(Gxc, Wc).T)
    return dict(Da=Da, Db=Db, Dc=Dc, Da_mu=W.T @ wh["mu_a"], Db_mu=Wb.T @ wh["mu_b"],
                Dc_mu=Wc.T @ wh["mu_c"], Wb=Wb, Wc=Wc)


def alpha_coeffs(alpha0):
    """Util.cpp:289-291: p0, p1, p2."""
    return ((alpha0 + 1.0) * (alpha0 + 2.0) / 2.0, alpha0 * alpha0,
            -alpha0 * (alpha0 + 1.0) / 2.0)


def tensor_decomp_batch(y, alpha0, phi0, min_iter=100, max_iter=10000, tol=TOLERANCE):
    """tensorDecom_alpha0, Util.cpp:131-184 (with tensor_form_* :187-206).

    Returns (lambda, phi, iterations, last_error)."""
    Da, Db, Dc = y["Da"], y["Db"], y["Dc"]
    a_mu, b_mu, c_mu = y["Da_mu"], y["Db_mu"], y["Dc_mu"]
    nx = Da.shape[1]
    inv_x = 1.0 / nx
    p_main = (alpha0 + 1.0) * (alpha0 + 2.0) / 2.0 * inv_x
    p_s1 = -alpha0 * (alpha0 + 1.0) / 2.0 * inv_x
    p_s0 = alpha0 * alpha0
    pair_ab, pair_ac, pair_bc = Da @ Db.T, Da @ Dc.T, Db @ Dc.T
    phi = np.array(phi0, dtype=np.float64, copy=True)
    it = 1
    while True:
        old = phi
        ZB, ZC = Db.T @ old, Dc.T @ old                       # n_X x k
        main = Da @ (ZB * ZC)
        mb, mc = old.T @ b_mu, old.T @ c_mu
        s1 = (np.outer(a_mu, np.einsum("ji,jl,li->i", old, pair_bc, old))
              + mb * (pair_ac @ old) + mc * (pair_ab @ old))
        s0 = np.outer(a_mu, mb * mc)
        new = p_main * main + p_s1 * s1 + p_s0 * s0
        lam = np.sum(new ** 2, axis=0) ** 1.5
        phi = new / np.linalg.norm(new, axis=0)
        err = np.nan
        if it >= min_iter:
            err = np.linalg.norm(phi - old)
            if err < tol or it > max_iter:
                break
        it += 1
    return lam, phi, it, err


def qr_pos(M):
    """Q of the QR factorisation M = Q R with R's diagonal non-negative: the
    per-step re-orthonormalisation of the reference's GPU tree
    (culaDeviceDgeqrfp + culaDeviceDorgqr, GPU/stpm.c:783-784, and the random
    start at GPU/stpm.c:1041-1064).  Householder QR (numpy/LAPACK dgeqrf),
    then the sign of each column of Q flipped where R's diagonal is negative,
    which gives the same Q as dgeqrfp; a zero diagonal keeps its column."""
    Q, R = np.linalg.qr(np.asarray(M, dtype=np.float64))
    s = np.sign(np.diag(R))
    s[s == 0] = 1.0
    return Q * s


def polar(M):
    """Orthonormal polar factor U V^T of M (M = U S V^T).  Not the
    reference's operator; kept as a named alternative orthonormalisation
    (stpm_online(..., orth="polar"))."""
    U, _, Vt = np.linalg.svd(M)
    return U @ Vt


def online_grad_terms(phi, y, nodes, alpha0):
    """Minibatch mean of the reference's per-sample second term
    (The_second_term, Util.cpp:286-304): column i = mean_x t_i(x)."""
    p0, p1, p2 = alpha_coeffs(alpha0)
    A, B, C = y["Da"][:, nodes], y["Db"][:, nodes], y["Dc"][:, nodes]
    ZA, ZB = phi.T @ A, phi.T @ B
    mA, mB = phi.T @ y["Da_mu"], phi.T @ y["Db_mu"]
    coef = p0 * ZA * ZB + p2 * (ZA * mB[:, None] + mA[:, None] * ZB)
    d = p1 * mA * mB + p2 * np.mean(ZA * ZB, axis=1)
    return C @ coef.T / A.shape[1] + np.outer(y["Dc_mu"], d)


def diff_loss_step(phi, y, nodes, alpha0, lr, theta):
    """Diff_Loss (Util.cpp:257-284) averaged over a minibatch:
    Phi - lr * (3 theta Phi (Phi^T Phi)^2 - 3 G)."""
    S = phi.T @ phi
    O = phi @ (S * S)
    G = online_grad_terms(phi, y, nodes, alpha0)
    return phi - lr * (3.0 * theta * O - 3.0 * G)


def loss_fwd(phi, y, nodes, alpha0, theta):
    """L(Phi) = theta sum_ij (phi_i.phi_j)^3 - 2 sum_i That(phi_i,phi_i,phi_i)."""
    p0, p1, p2 = alpha_coeffs(alpha0)
    ZA, ZB, ZC = (phi.T @ y[n][:, nodes] for n in ("Da", "Db", "Dc"))
    mA, mB, mC = (phi.T @ y[n] for n in ("Da_mu", "Db_mu", "Dc_mu"))
    t = p0 * ZA * ZB * ZC + p2 * (ZA * ZB * mC[:, None] + ZA * mB[:, None] * ZC
                                  + mA[:, None] * ZB * ZC)
    That = t.mean(axis=1) + p1 * mA * mB * mC
    S = phi.T @ phi
    return theta * np.sum(S ** 3) - 2.0 * np.sum(That)


def loss_bwd(phi, y, nodes, alpha0, theta):
    """Exact gradient dL/dPhi of loss_fwd (k x k)."""
    p0, p1, p2 = alpha_coeffs(alpha0)
    A, B, C = (y[n][:, nodes] for n in ("Da", "Db", "Dc"))
    ZA, ZB, ZC = phi.T @ A, phi.T @ B, phi.T @ C
    mA, mB, mC = (phi.T @ y[n] for n in ("Da_mu", "Db_mu", "Dc_mu"))
    b = A.shape[1]
    dZA = p0 * ZB * ZC + p2 * (ZB * mC[:, None] + mB[:, None] * ZC)
    dZB = p0 * ZA * ZC + p2 * (ZA * mC[:, None] + mA[:, None] * ZC)
    dZC = p0 * ZA * ZB + p2 * (ZA * mB[:, None] + mA[:, None] * ZB)
    dmA = p2 * np.mean(ZB * ZC, axis=1) + p1 * mB * mC
    dmB = p2 * np.mean(ZA * ZC, axis=1) + p1 * mA * mC
    dmC = p2 * np.mean(ZA * ZB, axis=1) + p1 * mA * mB
    dT = ((A @ dZA.T + B @ dZB.T + C @ dZC.T) / b + np.outer(y["Da_mu"], dmA)
          + np.outer(y["Db_mu"], dmB) + np.outer(y["Dc_mu"], dmC))
    S = phi.T @ phi
    return 6.0 * theta * phi @ (S * S) - 2.0 * dT


def stpm_minibatches(nx, minibatch):
    return [np.arange(s, min(s + minibatch, nx)) for s in range(0, nx, minibatch)]


def tensor_values(phi, y, alpha0):
    """lambda_i = That(phi_i, phi_i, phi_i) over all of X."""
    nodes = np.arange(y["Da"].shape[1])
    G = online_grad_terms(phi, y, nodes, alpha0)
    return np.einsum("ji,ji->i", phi, G)


def stpm_online(y, alpha0, phi0, sweeps, minibatch, lr0=1.0, theta=0.5, adjoint=False,
                orth="qr"):
    """Minibatch STPM: per step Phi <- qr_pos(Phi - beta_t (3 theta O - 3 G))
    with O = Phi (Phi^T Phi)^.2 (Diff_Loss, Util.cpp:257-284, averaged over
    the minibatch; the same update as GPU/stpm.c:649-691 with the learning
    rate of the BASELINE schedule), re-orthonormalised every step by QR with
    a non-negative R diagonal as GPU/stpm.c:774-786 does; beta_t = lr0/(1+t).
    adjoint=True uses half the exact gradient of loss_fwd instead of
    3 theta O - 3 G.  orth="polar" replaces the QR by the polar factor (not
    the reference's operator).
    Returns (lambda, phi, steps) with lambda_i = That(phi_i,phi_i,phi_i) > 0."""
    orthonormalise = {"qr": qr_pos, "polar": polar}[orth]
    nx = y["Da"].shape[1]
    phi = np.array(phi0, dtype=np.float64, copy=True)
    t = 0
    batches = stpm_minibatches(nx, minibatch)
    for _ in range(sweeps):
        for nodes in batches:
            beta = lr0 / (1.0 + t)
            if adjoint:
                step = 0.5 * loss_bwd(phi, y, nodes, alpha0, theta)
            else:
                S = phi.T @ phi
                step = 3.0 * theta * (phi @ (S * S)) - 3.0 * online_grad_terms(phi, y, nodes,
                                                                                 alpha0)
            phi = orthonormalise(phi - beta * step)
            t += 1
    if t == 0:
        phi = orthonormalise(phi)
    lam = tensor_values(phi, y, alpha0)
    sgn = np.where(lam < 0, -1.0, 1.0)
    return lam * sgn, phi * sgn, t


def norm_prob_matrix(P):
    """normProbMatrix / normProbVector, Probability.cpp:33-121, column-wise."""
    P = np.asarray(P, dtype=np.float64)
    pos = np.where(P > 0, P, 0.0).sum(axis=0)
    neg = np.where(P > 0, 0.0, P).sum(axis=0)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = np.where(np.abs(pos) < np.abs(neg), -P / np.abs(neg), P / np.where(pos == 0, 1, np.abs(pos)))
    out = np.maximum(out, 0.0)
    zero = ~np.any(P != 0, axis=0)
    out[:, zero] = P[:, zero]
    return out


def postprocess(Gxa, Gba, Gca, wh, lam, phi, tol=TOLERANCE):
    """CommunityDetection.cpp:98-139: returns (pi_raw, pi) k x (n_X+n_A+n_B+n_C)."""
    P_A = wh["W"] @ (phi * pinv_vector(lam, tol))          # (diag(1/lam) Phi^T W^T)^T
    pi_x = _mm(Gxa, P_A).T
    pi_b = _mm(Gba, P_A).T
    pi_c = _mm(Gca, P_A).T
    P_A2 = wh["Zb2"].T @ (wh["Zb1"].T @ P_A)
    pi_a = _mm(Gba.T.tocsr(), P_A2).T
    raw = np.concatenate([np.asarray(m) for m in (pi_x, pi_a, pi_b, pi_c)], axis=1)
    return raw, norm_prob_matrix(raw)


def community_sets(pi, tau):
    return pi > tau


# ---- file contract and ground-truth evaluation ------------------------------

def read_coo_reference(text, n_rows, n_cols, datatype=0):
    """read_G_sparse (IOfn.cpp:21-54) on a COO text: the while(!feof) loop of
    fscanf("%lf") reads "row col" (datatype 0) or "row col value" per pass.  A
    read that meets the end of the file leaves its variable unchanged and sets
    EOF; a number that ends exactly at the end of the file also sets EOF.  So
    after the last complete triplet one more pass pushes the previous triplet
    again unless the last number ended the file, and a trailing partial
    triplet is completed with the previous values.  Triplets are summed
    (setFromTriplets), then prune(1e-6) keeps |v| > 1e-18.  Returns CSR.
    (Files shorter than one triplet and non-numbers are undefined behaviour in
    the reference; they are rejected here with ValueError.)"""
    toks, ends = [], []
    for m in __import__("re").finditer(r"\S+", text):
        toks.append(float(m.group(0)))
        ends.append(m.end())
    per = 3 if datatype == 1 else 2
    if len(toks) < per:
        raise ValueError("shorter than one triplet")
    last_eof = ends[-1] == len(text)
    trip, cur, i, eof = [], [None] * per, 0, False
    while not eof:
        for f in range(per):
            if i < len(toks):
                cur[f] = toks[i]
                if i == len(toks) - 1 and last_eof:
                    eof = True
                i += 1
            else:
                eof = True
        trip.append(tuple(cur))
    r = np.array([int(t[0] - 1) for t in trip])
    c = np.array([int(t[1] - 1) for t in trip])
    v = np.array([t[2] if per == 3 else 1.0 for t in trip])
    if (r < 0).any() or (r >= n_rows).any() or (c < 0).any() or (c >= n_cols).any():
        raise ValueError("index out of range")
    m = sp.coo_matrix((v, (r, c)), shape=(n_rows, n_cols)).tocsr()
    m.sum_duplicates()
    m.data[np.abs(m.data) <= 1e-18] = 0.0
    m.eliminate_zeros()
    return m


def _betacf(a, b, x):
    """Continued fraction of the incomplete beta function by the modified
    Lentz method (Numerical Recipes 6.4), as Pvalue.cpp:121-185 evaluates it:
    stop when |del - 1| <= 3e-7, FPMIN 1e-30."""
    fpmin, eps = 1e-30, 3e-7
    qab, qap, qam = a + b, a + 1.0, a - 1.0
    c, d = 1.0, 1.0 - qab * x / qap
    d = fpmin if abs(d) < fpmin else d
    d = 1.0 / d
    h = d
    m = 0
    while m <= 100000:
        m += 1
        m2 = 2 * m
        aa = m * (b - m) * x / ((qam + m2) * (a + m2))
        d = 1.0 + aa * d
        d = fpmin if abs(d) < fpmin else d
        c = 1.0 + aa / c
        c = fpmin if abs(c) < fpmin else c
        d = 1.0 / d
        h = h * d * c
        aa = -(a + m) * (qab + m) * x / ((a + m2) * (qap + m2))
        d = 1.0 + aa * d
        d = fpmin if abs(d) < fpmin else d
        c = 1.0 + aa / c
        c = fpmin if abs(c) < fpmin else c
        d = 1.0 / d
        dl = d * c
        h = h * dl
        if abs(dl - 1.0) <= eps:
            return h
    raise ValueError("betacf did not converge")


# Lanczos coefficients of Numerical Recipes' gammln (6.1), Pvalue.cpp:189-204
_GAMMLN_COF = (76.18009173, -86.50532033, 24.01409822, -1.231739516, 0.120858003e-2, -0.536382e-5)


def _gammln(xx):
    x = xx - 1.0
    tmp = x + 5.5
    tmp -= (x + 0.5) * np.log(tmp)
    ser = 1.0
    for cof in _GAMMLN_COF:
        x += 1.0
        ser += cof / x
    return -tmp + np.log(2.50662827465 * ser)


def _betainc(a, b, x):
    """Pvalue.cpp:206-230 (regularised incomplete beta)."""
    if x == 0 or x == 1:
        bt = 0.0
    else:
        bt = np.exp(_gammln(a + b) - _gammln(a) - _gammln(b) + a * np.log(x) + b * np.log(1.0 - x))
    if x < (a + 1.0) / (a + b + 2.0):
        return bt * _betacf(a, b, x) / a
    return 1.0 - bt * _betacf(b, a, 1.0 - x) / b


def pvalue_stats(x, y):
    """(correlation, t statistic, p-value) of Calculate_Correlation /
    Calculate_Tstat / Calculate_Pvalue (Pvalue.cpp:85-235): population
    moments, t = r sqrt((n-2)/(1-r^2)), two-sided p from the incomplete beta
    function with n-2 degrees of freedom.  The reference's branch order is
    kept: p is 0.5 (so 1 is returned) unless n-2 != 1, n-2 <= 1e7 and neither
    t is NaN nor n-2 <= 0."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(x)
    mx, my = x.sum() / n, y.sum() / n
    cov = ((x - mx) * (y - my)).sum() / n
    sx = np.sqrt(((x - mx) ** 2).sum() / n)
    sy = np.sqrt(((y - my) ** 2).sum() / n)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = cov / (sx * sy)
        t_raw = r * np.sqrt((n - 2) / (1 - r * r))
    t = -abs(t_raw)
    dof = float(n - 2)
    nans = np.isnan(t) or dof <= 0
    if dof != 1 and dof <= 1e7 and not nans:
        p = 0.5 * _betainc(0.5 * dof, 0.5, dof / (dof + t * t))
        if t > 0:
            p = 1 - p
    else:
        p = 0.5
    return float(r), float(t_raw), float(2 * p)
