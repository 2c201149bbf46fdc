"""The formulation of the device tabulation of the diatomic two-electron
primitives, restated in numpy and checked against the host tabulation on
the CPU (the CUDA kernels themselves are checked against the host tables in
tests/test_gpu_diatomic_tabulation.py).

What the restatement fixes, as the device kernels compute it
(helfem_gb300/csrc/cuda/dtab_fp64.cu):
* the in-element points in reference coordinates: on elements after the
  first, x = (1 + x_q)(1 + x_r)/2 - 1 for the inner points; on the first
  (mu = mu_1 t^3), 2 t^3 - 1 and t^3 (1 + x_r) - 1;
* the kernel before symmetrisation as one product R = O^T I over the outer
  points, with the two channels stacked along the unique primitive pairs;
* the two-channel kernel read from R, W(i, j) = +-(R(c_i, c_j) + R(c_j, c_i)),
  negative across channels;
* the sign-carrying pivoted factor with the host's pivot rule.
The reconstructed kernels must agree with the host tabulation's to 1e-13 of
each kernel's largest entry (src/diatomic/basis.cpp:1432-1545).
"""
import numpy as np

import helfem_gb300 as hg
from oracle.diatomic import legendre_pq
from oracle.tabulate import gauss_legendre, lip_eval, lobatto


def restated_kernels(d, elems, ilms, thresh=1e-12):
    dims = d.dims
    nn, nrad, Lmax = dims["nnodes"], dims["nrad"], dims["Lmax"]
    n2, npr = nn * nn, nn * (nn + 1) // 2
    N = 2 * n2
    lm = [d.tables(0, i, 0)[:2] for i in range(dims["nlm"])]
    Mtop = max(M for _, M in lm)
    xn, _ = lobatto(nn)
    xo, wo = gauss_legendre(64)
    xi, wi = gauss_legendre(64)
    t = 0.5 * (xo + 1.0)
    B1 = {False: lip_eval(xo, xn, 0), True: lip_eval(2.0 * t ** 3 - 1.0, xn, 0)}
    r2 = {False: (0.5 * (1.0 + xo)[:, None] * (1.0 + xi)[None, :] - 1.0).ravel(),
          True: ((t ** 3)[:, None] * (1.0 + xi)[None, :] - 1.0).ravel()}
    B2 = {k: lip_eval(v, xn, 0) for k, v in r2.items()}
    pa = np.concatenate([np.arange(b + 1) for b in range(nn)])
    pb = np.concatenate([np.full(b + 1, b) for b in range(nn)])
    # row i of W -> (channel, index into R)
    ch = np.arange(N) // n2
    a, b = (np.arange(N) % n2) % nn, (np.arange(N) % n2) // nn
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    cidx = lo + hi * (hi + 1) // 2 + ch * npr
    sign = np.where(ch[:, None] != ch[None, :], -1.0, 1.0)
    bval = d._bval
    out = {}
    for e in elems:
        first = e == 0
        ok = np.array([e * (nn - 1) + p < nrad for p in range(nn)])
        okp = (ok[pa] & ok[pb]).astype(float)
        mus, mue = bval[e], bval[e + 1]
        if first:
            mu1, w1 = mus + (mue - mus) * t ** 3, 0.5 * wo * 3.0 * (mue - mus) * t ** 2
        else:
            sf, mid = 0.5 * (mue - mus), 0.5 * (mue + mus)
            mu1, w1 = mid + sf * xo, sf * wo
        h = 0.5 * (mu1 - mus)
        mu2 = mus + h[:, None] * (xi[None, :] + 1.0)  # [q, r]
        w2 = h[:, None] * wi[None, :]
        P2, _ = legendre_pq(Lmax, Mtop, mu2.ravel())
        _, Q1 = legendre_pq(Lmax, Mtop, mu1)
        BB1 = B1[first][:, pa] * B1[first][:, pb] * okp                      # [q, k]
        BB2 = (B2[first][:, pa] * B2[first][:, pb] * okp).reshape(64, 64, -1)  # [q, r, k]
        for ilm in ilms:
            L, M = lm[ilm]
            wr0 = (w2 * np.sinh(mu2)) * P2[M, L].reshape(64, 64)
            wr2 = wr0 * np.cosh(mu2) ** 2
            I = np.concatenate([np.einsum("qr,qrk->qk", wr0, BB2), np.einsum("qr,qrk->qk", wr2, BB2)], axis=1)
            wq0 = w1 * np.sinh(mu1) * Q1[M, L]
            O = np.concatenate([wq0[:, None] * BB1, (wq0 * np.cosh(mu1) ** 2)[:, None] * BB1], axis=1)
            R = O.T @ I
            Rc = R[np.ix_(cidx, cidx)]
            W = sign * (Rc + Rc.T)
            dg = np.diag(W).copy()
            dmax0 = np.abs(dg).max()
            cols, sg = [], []
            for _ in range(N):
                piv = int(np.argmax(np.abs(dg)))
                dp = dg[piv]
                if dmax0 <= 0.0 or abs(dp) <= thresh * dmax0:
                    break
                s = 1.0 if dp >= 0.0 else -1.0
                col = W[:, piv].copy()
                for c, sq in zip(cols, sg):
                    col -= sq * c[piv] * c
                col /= np.sqrt(abs(dp))
                dg -= s * col * col
                dg[piv] = 0.0
                cols.append(col)
                sg.append(s)
            Bm = np.array(cols).T
            out[(ilm, e)] = (Bm * np.array(sg)) @ Bm.T, Bm.shape[1]
    return out


def test_device_formulation_matches_host_tables():
    # heteronuclear, m up to 1, 5-node elements; the first and the last
    # element (the mu = mu_1 t^3 map and the dropped outermost function) and
    # one in between
    d = hg.Diatomic.from_grid(2, 1, 1.46, 4, [2, 1], nnodes=5, host_only=True)
    nlm, nel = d.dims["nlm"], d.dims["nel"]
    res = restated_kernels(d, [0, 1, nel - 1], range(0, nlm, 2))
    worst = 0.0
    for (ilm, e), (W, r) in res.items():
        _, _, Bh, sh = d.tables(4, ilm, e)
        Wh = (Bh * sh) @ Bh.T
        assert r == Bh.shape[1], (ilm, e)
        worst = max(worst, float(np.abs(W - Wh).max() / np.abs(Wh).max()))
    assert worst <= 1e-13, worst
