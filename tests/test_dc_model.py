"""A scalar restatement of the divide-and-conquer quadrature kernel
(tridiag_dc_kernel: the same torn leaves, merge levels, deflation, secular
iteration, Loewner vectors and merge order) against numpy's eigh.  No GPU.

It checks the algorithm the kernel implements on the CPU: eigenvalues to
1e-12 of the spectral radius and Gauss quadratures sum_i g(lambda_i) s_1i^2 to
1e-12 on Gaussian, Wilkinson, glued, split, tiny-coupling and zero
tridiagonals.

``dc_full`` runs the same merges carrying whole eigenvector columns instead of
their first and last rows (tridiag_dcv_kernel, the eigenvectors of the
gradient's Daleckii-Krein term): S^T S = I and S diag(lambda) S^T = T to
1e-12 k on the same spectra.
"""

import math

import numpy as np
import pytest

EPS = np.finfo(np.float64).eps


def _quad_root(c, P1, P2, s1, s2):
    # root in (P1, P2) of c + s1/(P1 - x) + s2/(P2 - x) = 0
    a1 = c * (P1 + P2) + s1 + s2
    a0 = c * P1 * P2 + s1 * P2 + s2 * P1
    sq = math.sqrt(max(a1 * a1 - 4.0 * c * a0, 0.0))
    return 2.0 * a0 / (a1 + sq) if a1 > 0 else (a1 - sq) / (2.0 * c)


def _quad_step(c, A, B, s1, s2, f):
    a1 = c * (A + B) + s1 + s2
    a0 = A * B * f
    sq = math.sqrt(max(a1 * a1 - 4.0 * c * a0, 0.0))
    if a1 > 0:
        return 2.0 * a0 / (a1 + sq)
    return (a1 - sq) / (2.0 * c) if c != 0 else math.nan


def _quad_step_right(c, A0, A, s0, s1, f):
    a1 = c * (A0 + A) + s0 + s1
    a0 = A0 * A * f
    sq = math.sqrt(max(a1 * a1 - 4.0 * c * a0, 0.0))
    return (a1 + sq) / (2.0 * c) if a1 >= 0 else 2.0 * a0 / (a1 - sq)


def _secular(P, ZZ, mk, j, rho, upper):
    """Root j as (offset x, origin o); the kernel's dc_secular_root."""
    ir = 1.0 / rho
    last = j + 1 >= mk
    lo_pole = P[j]
    hi_pole = upper if last else P[j + 1]
    xma = 0.5 * (lo_pole + hi_pole)
    fmid = ir + sum(ZZ[i] / (P[i] - xma) for i in range(mk))
    zzj, zzj1 = ZZ[j], (0.0 if last else ZZ[j + 1])
    two_below = last and mk > 1
    zzjm = ZZ[j - 1] if two_below else 0.0
    o = j + 1 if (not last and fmid < 0.0) else j
    base = P[o]
    lo, hi = lo_pole - base, hi_pole - base
    P1 = P[j] - base
    P2 = hi if last else P[j + 1] - base
    P0 = P[j - 1] - base if two_below else 0.0
    xm = 0.5 * (lo + hi)
    if mk == 1:
        x = rho * zzj
    elif last:
        c = fmid - zzj / (P[j] - xma) - zzjm / (P[j - 1] - xma)
        x = xm + _quad_step_right(c, P0 - xm, P1 - xm, zzjm, zzj, fmid) if c > 0 else xm
    else:
        c = fmid - zzj / (P[j] - xma) - zzj1 / (P[j + 1] - xma)
        x = _quad_root(c, P1, P2, zzj, zzj1)
    if not (lo < x < hi):
        x = xm
    m0, m1 = (j - 1 if two_below else j), (j if last else j + 1)
    for _ in range(128):
        rs = drs = ab = 0.0
        for i in range(mk):
            if m0 <= i <= m1:
                continue
            inv = 1.0 / ((P[i] - base) - x)
            t = ZZ[i] * inv
            rs += t
            drs += t * inv
            ab += abs(t)
        A, B, A0 = P1 - x, P2 - x, P0 - x
        tj = zzj / A
        tj1 = 0.0 if last else zzj1 / B
        tjm = zzjm / A0 if two_below else 0.0
        f = ir + rs + tj + tj1 + tjm
        sab = ab + abs(tj) + abs(tj1) + abs(tjm)
        if f > 0:
            hi = x
        else:
            lo = x
        if abs(f) <= EPS * mk * (ir + sab) or hi - lo <= 2.0 * EPS * max(abs(lo), abs(hi)):
            return x, o, True
        if last and mk == 1:
            eta = A + zzj * rho
        elif last:
            c = ir + rs - drs * A0
            eta = _quad_step_right(c, A0, A, zzjm + drs * A0 * A0, zzj, f) if c > 0 else math.nan
        elif o == j:
            eta = _quad_step(ir + rs - drs * B, A, B, zzj, zzj1 + drs * B * B, f)
        else:
            eta = _quad_step(ir + rs - drs * A, A, B, zzj + drs * A * A, zzj1, f)
        if abs(eta) <= 2.0 * EPS * abs(x):
            return x, o, True
        xn = x + eta
        x = xn if lo < xn < hi else 0.5 * (lo + hi)
    return x, o, False


def dc_first_rows(d, e):
    """Eigenvalues (ascending) and squared first eigenvector components."""
    k = len(d)
    LAM = np.array([d[i] - (e[i - 1] if i > 0 else 0.0) - (e[i] if i + 1 < k else 0.0) for i in range(k)])
    FR, LR = np.ones(k), np.ones(k)
    ok = True
    w = 1
    while w < k:
        for a in range(0, k - w, 2 * w):  # merges of this level
            mid, hi = a + w, min(a + 2 * w, k)
            rho = e[mid - 1]
            sg = -1.0 if rho < 0 else 1.0
            rho = abs(rho)
            tol = 8.0 * EPS * max(abs(LAM[a]), abs(LAM[mid - 1]), abs(LAM[mid]), abs(LAM[hi - 1]), 2.0 * rho)
            # sorted merge of the halves (negated when rho < 0), with deflation
            items = [(sg * LAM[i], LR[i], FR[i], 0.0) for i in range(a, mid)]
            items += [(sg * LAM[i], FR[i], 0.0, LR[i]) for i in range(mid, hi)]
            items.sort(key=lambda t: t[0])
            D, Z, F, L, dfl = [], [], [], [], []
            zs = 0.0
            for dv, z, f, l in items:
                if rho * abs(z) <= tol:
                    dfl.append((dv, f, l))
                    continue
                zs += z * z
                if D and dv - D[-1] <= tol:  # close poles: rotate, drop the earlier
                    r = math.hypot(Z[-1], z)
                    c, s = z / r, Z[-1] / r
                    dfl.append((D[-1], c * F[-1] - s * f, c * L[-1] - s * l))
                    D[-1], Z[-1], F[-1], L[-1] = dv, r, s * F[-1] + c * f, s * L[-1] + c * l
                else:
                    D.append(dv), Z.append(z), F.append(f), L.append(l)
            dfl.sort(key=lambda t: t[0])
            mk = len(D)
            out = []
            if mk:
                upper = D[-1] + rho * zs * (1.0 + 16.0 * EPS) + 16.0 * EPS * abs(D[-1])
                ZZ = [z * z for z in Z]
                roots = []
                for j in range(mk):
                    x, o, conv = _secular(D, ZZ, mk, j, rho, upper)
                    ok &= conv
                    roots.append((x, o))
                zh = []
                for i in range(mk):  # Loewner
                    prod = ((D[roots[mk - 1][1]] - D[i]) + roots[mk - 1][0]) / rho
                    for j in range(mk - 1):
                        prod *= ((D[roots[j][1]] - D[i]) + roots[j][0]) / (D[j if j < i else j + 1] - D[i])
                    zh.append(math.copysign(math.sqrt(max(prod, 0.0)), Z[i]))
                for j in range(mk):
                    x, o = roots[j]
                    u = np.array([zh[i] / ((D[i] - D[o]) - x) for i in range(mk)])
                    u /= np.linalg.norm(u)
                    out.append((D[o] + x, float(np.dot(F, u)), float(np.dot(L, u))))
            merged = sorted(out + dfl, key=lambda t: t[0])
            if sg < 0:
                merged = [(-v, f, l) for v, f, l in reversed(merged)]
            for t, (v, f, l) in enumerate(merged):
                LAM[a + t], FR[a + t], LR[a + t] = v, f, l
        w *= 2
    return LAM, FR * FR, ok


def _case(kind, k, rng):
    if kind == "normal":
        return rng.standard_normal(k), rng.standard_normal(k - 1)
    if kind == "wilkinson":
        return np.abs(np.arange(k) - k // 2).astype(float), np.ones(k - 1)
    if kind == "glued":
        d = np.resize(np.abs(np.arange(7) - 3).astype(float), k)
        e = np.ones(k - 1)
        e[6::7] = 1e-10
        return d, e
    if kind == "split":
        e = np.zeros(k - 1)
        e[::3] = 1.0
        return np.ones(k), e
    if kind == "tiny":
        return rng.standard_normal(k), rng.standard_normal(k - 1) * 10.0 ** rng.integers(-18, 0, k - 1)
    if kind == "negative":
        return rng.uniform(1, 3, k), -rng.uniform(0.1, 0.5, k - 1)
    return np.zeros(k), np.zeros(k - 1)


@pytest.mark.parametrize("kind", ["normal", "wilkinson", "glued", "split", "tiny", "negative", "zero"])
@pytest.mark.parametrize("k", [1, 2, 5, 16, 17, 33])
def test_dc_model_matches_eigh(kind, k):
    rng = np.random.default_rng(100 * sum(map(ord, kind)) + k)
    d, e = _case(kind, k, rng) if k > 1 else (rng.standard_normal(1), np.zeros(0))
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    w0, S0 = np.linalg.eigh(T)
    lam, fsq, ok = dc_first_rows(d, e)
    assert ok
    scale = max(np.abs(w0).max(), 1e-300)
    np.testing.assert_allclose(lam, w0, rtol=0, atol=1e-12 * scale)
    for g in (lambda x: np.exp(-x / scale), lambda x: np.sin(3 * x / scale)):
        assert abs(np.sum(g(lam) * fsq) - np.sum(g(w0) * S0[0] ** 2)) <= 1e-12


def dc_full(d, e):
    """Eigenvalues (ascending) and eigenvectors (columns) by the same merges."""
    k = len(d)
    LAM = np.array([d[i] - (e[i - 1] if i > 0 else 0.0) - (e[i] if i + 1 < k else 0.0) for i in range(k)])
    S = np.eye(k)  # columns: eigenvectors of the current block-diagonal problem
    ok = True
    w = 1
    while w < k:
        for a in range(0, k - w, 2 * w):
            mid, hi = a + w, min(a + 2 * w, k)
            rho = e[mid - 1]
            sg = -1.0 if rho < 0 else 1.0
            rho = abs(rho)
            tol = 8.0 * EPS * max(abs(LAM[a]), abs(LAM[mid - 1]), abs(LAM[mid]), abs(LAM[hi - 1]), 2.0 * rho)
            # z: the last row of the upper block's vectors, the first row of the lower block's
            cols = [(sg * LAM[i], S[mid - 1, i], S[a:hi, i].copy()) for i in range(a, mid)]
            cols += [(sg * LAM[i], S[mid, i], S[a:hi, i].copy()) for i in range(mid, hi)]
            cols.sort(key=lambda t: t[0])
            D, Z, V, dfl = [], [], [], []
            zs = 0.0
            for dv, z, v in cols:
                if rho * abs(z) <= tol:
                    dfl.append((dv, v))
                    continue
                zs += z * z
                if D and dv - D[-1] <= tol:  # close poles: the same rotation, on whole columns
                    r = math.hypot(Z[-1], z)
                    c, s = z / r, Z[-1] / r
                    dfl.append((D[-1], c * V[-1] - s * v))
                    D[-1], Z[-1], V[-1] = dv, r, s * V[-1] + c * v
                else:
                    D.append(dv), Z.append(z), V.append(v)
            mk = len(D)
            out = []
            if mk:
                upper = D[-1] + rho * zs * (1.0 + 16.0 * EPS) + 16.0 * EPS * abs(D[-1])
                ZZ = [z * z for z in Z]
                roots = []
                for j in range(mk):
                    x, o, conv = _secular(D, ZZ, mk, j, rho, upper)
                    ok &= conv
                    roots.append((x, o))
                zh = []
                for i in range(mk):  # Loewner
                    prod = ((D[roots[mk - 1][1]] - D[i]) + roots[mk - 1][0]) / rho
                    for j in range(mk - 1):
                        prod *= ((D[roots[j][1]] - D[i]) + roots[j][0]) / (D[j if j < i else j + 1] - D[i])
                    zh.append(math.copysign(math.sqrt(max(prod, 0.0)), Z[i]))
                Vm = np.stack(V, axis=1)
                for j in range(mk):
                    x, o = roots[j]
                    u = np.array([zh[i] / ((D[i] - D[o]) - x) for i in range(mk)])
                    out.append((D[o] + x, Vm @ (u / np.linalg.norm(u))))
            merged = sorted(out + dfl, key=lambda t: t[0])
            if sg < 0:
                merged = [(-v, vec) for v, vec in reversed(merged)]
            for t, (v, vec) in enumerate(merged):
                LAM[a + t] = v
                S[:, a + t] = 0.0
                S[a:hi, a + t] = vec
        w *= 2
    return LAM, S, ok


@pytest.mark.parametrize("kind", ["normal", "wilkinson", "glued", "split", "tiny", "negative", "zero"])
@pytest.mark.parametrize("k", [1, 2, 17, 48, 100])
def test_dc_full_vectors_match_eigh(kind, k):
    rng = np.random.default_rng(100 * sum(map(ord, kind)) + k)
    d, e = _case(kind, k, rng) if k > 1 else (rng.standard_normal(1), np.zeros(0))
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    lam, S, ok = dc_full(d, e)
    assert ok
    scale = max(np.abs(np.linalg.eigvalsh(T)).max(), 1e-300)
    np.testing.assert_allclose(lam, np.linalg.eigvalsh(T), rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(S.T @ S, np.eye(k), atol=1e-12 * k)
    np.testing.assert_allclose((S * lam) @ S.T, T, atol=1e-12 * k * scale)


# ---------------------------------------------------------------------------
# The eigenvector kernel's own index arithmetic (column-index array CI, in-place
# close-pole rotations, the S2 staging and the column map O), run phase by
# phase with the threads of a phase one after another: a phase's threads touch
# disjoint entries, so the order does not matter.  Roots come from the scalar
# secular solver above; everything else follows the CUDA source line by line.

def dcv_kernel_phases(H):
    """tridiag_dcv_kernel phase by phase, threads run one after another."""
    k = H.shape[0]
    EO = np.array([0.5 * (H[i, i + 1] + H[i + 1, i]) if i + 1 < k else 0.0 for i in range(k)])
    LAM = np.array([H[i, i] - (EO[i - 1] if i > 0 else 0.0) - EO[i] for i in range(k)])
    S = np.zeros(k * k); S2 = np.zeros(k * k); U = np.zeros(k * k)
    for i in range(k): S[i * k + i] = 1.0
    D = np.zeros(k); Z = np.zeros(k); X = np.zeros(k); NF = np.zeros(k)
    CI = np.zeros(k, dtype=int); O = np.zeros(k, dtype=int)
    kh = (k + 1) // 2
    MS = np.zeros(kh, dtype=int); RH = np.zeros(kh); UB = np.zeros(kh)
    FLIP = 1 << 30
    ok = True
    s = 0
    while (1 << s) < k:
        w = 1 << s; span = 2 * w; nm = (k - w - 1) // span + 1
        # A
        for q in range(nm):
            a = q * span; mid = a + w; hi = min(a + span, k)
            rho = EO[mid - 1]; flip = rho < 0.0; sg = -1.0 if flip else 1.0; rho = abs(rho)
            maxabs = max(abs(LAM[a]), abs(LAM[mid - 1]), abs(LAM[mid]), abs(LAM[hi - 1]))
            tol = 8.0 * EPS * max(maxabs, 2.0 * rho)
            n1, n2 = mid - a, hi - mid
            c1 = c2 = 0; kp = a; dp = hi; zs = 0.0
            for t in range(a, hi):
                if c1 == n1: take1 = False
                elif c2 == n2: take1 = True
                else: take1 = sg * LAM[mid - 1 - c1 if flip else a + c1] <= sg * LAM[hi - 1 - c2 if flip else mid + c2]
                if take1:
                    col = mid - 1 - c1 if flip else a + c1; z = S[col * k + (mid - 1)]; c1 += 1
                else:
                    col = hi - 1 - c2 if flip else mid + c2; z = S[col * k + mid]; c2 += 1
                d = sg * LAM[col]
                if rho * abs(z) <= tol:
                    dp -= 1; D[dp] = d; CI[dp] = col; continue
                zs = zs + z * z
                if kp > a and d - D[kp - 1] <= tol:
                    zp = Z[kp - 1]; r = math.hypot(zp, z); c = z / r; sn = zp / r; cp = CI[kp - 1]
                    for t2 in range(a, hi):
                        vp, vc = S[cp * k + t2], S[col * k + t2]
                        S[cp * k + t2] = c * vp - sn * vc
                        S[col * k + t2] = sn * vp + c * vc
                    dp -= 1; D[dp] = D[kp - 1]; CI[dp] = cp
                    D[kp - 1] = d; Z[kp - 1] = r; NF[kp - 1] = r * r; CI[kp - 1] = col
                else:
                    D[kp] = d; Z[kp] = z; NF[kp] = z * z; CI[kp] = col; kp += 1
            u, v = dp, hi - 1
            while u < v:
                D[u], D[v] = D[v], D[u]; CI[u], CI[v] = CI[v], CI[u]; u += 1; v -= 1
            for u in range(dp + 1, hi):
                dv, cv = D[u], CI[u]; v = u - 1
                while v >= dp and D[v] > dv:
                    D[v + 1] = D[v]; CI[v + 1] = CI[v]; v -= 1
                D[v + 1] = dv; CI[v + 1] = cv
            mk = kp - a
            MS[q] = mk | (FLIP if flip else 0); RH[q] = rho
            UB[q] = D[kp - 1] + rho * zs * (1.0 + 16.0 * EPS) + 16.0 * EPS * abs(D[kp - 1]) if mk > 0 else 0.0
        # B, C, D (roots via the model's secular solver, zhat, U)
        for q in range(nm):
            a = q * span; mk = MS[q] & (FLIP - 1)
            P = D[a:a + mk].copy(); ZZ = NF[a:a + mk].copy()
            xs = []
            for j in range(mk):
                x, o, conv = _secular(list(P), list(ZZ), mk, j, RH[q], UB[q]); ok &= conv
                xs.append((x, o)); X[a + j] = x; O[a + j] = o
            for i in range(mk):
                di = P[i]
                prod = ((P[O[a + mk - 1]] - di) + X[a + mk - 1]) / RH[q]
                for j in range(mk - 1):
                    prod *= ((P[O[a + j]] - di) + X[a + j]) / (P[j if j < i else j + 1] - di)
                Z[a + i] = math.copysign(math.sqrt(max(prod, 0.0)), Z[a + i])
            for j in range(mk):
                r = a + j; ox = P[O[r]]; x = X[r]
                us = [Z[a + i] / ((P[i] - ox) - x) for i in range(mk)]
                rn = 1.0 / math.sqrt(sum(u * u for u in us))
                for i in range(mk): U[r * k + i] = us[i] * rn
                X[r] = ox + x
        # D'
        for idx in range(nm * span * span):
            q = idx // (span * span); rem = idx - q * span * span; j = rem // span; tt = rem - j * span
            a = q * span; hi = min(a + span, k); c = a + j; t = a + tt
            if c >= hi or t >= hi: continue
            mk = MS[q] & (FLIP - 1)
            if j < mk:
                acc = 0.0
                for i in range(mk): acc += U[c * k + i] * S[CI[a + i] * k + t]
                S2[c * k + t] = acc
            else:
                S2[c * k + t] = S[CI[c] * k + t]
        # E
        for q in range(nm):
            a = q * span; hi = min(a + span, k); mk = MS[q] & (FLIP - 1); flip = (MS[q] & FLIP) != 0
            sg = -1.0 if flip else 1.0; c1 = a; c2 = a + mk
            for t in range(hi - a):
                if c1 < a + mk and (c2 >= hi or X[c1] <= D[c2]):
                    v = X[c1]; src = c1; c1 += 1
                else:
                    v = D[c2]; src = c2; c2 += 1
                pos = hi - 1 - t if flip else a + t
                LAM[pos] = sg * v; O[pos] = src
        for idx in range(nm * span * span):
            q = idx // (span * span); rem = idx - q * span * span; j = rem // span; tt = rem - j * span
            a = q * span; hi = min(a + span, k); c = a + j; t = a + tt
            if c >= hi or t >= hi: continue
            S[c * k + t] = S2[O[c] * k + t]
        s += 1
    Sout = S.reshape(k, k).T.copy()  # Sb[row*k + j] = S[j*k + row]
    return LAM, Sout, ok


@pytest.mark.parametrize("kind", ["normal", "wilkinson", "glued", "split", "tiny", "negative", "zero"])
@pytest.mark.parametrize("k", [16, 20, 33, 48, 64])
def test_dcv_kernel_phases_match_eigh(kind, k):
    rng = np.random.default_rng(1000 * k + sum(map(ord, kind)))
    d, e = _case(kind, k, rng)
    H = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    lam, S, ok = dcv_kernel_phases(H)
    assert ok
    w0 = np.linalg.eigvalsh(H)
    scale = max(np.abs(w0).max(), 1e-300)
    np.testing.assert_allclose(lam, w0, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(S.T @ S, np.eye(k), atol=1e-12 * k)
    np.testing.assert_allclose((S * lam) @ S.T, H, atol=1e-12 * k * scale)
