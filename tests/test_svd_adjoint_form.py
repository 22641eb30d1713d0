"""The FP32 adjoint's algebra, checked in FP64 numpy (no GPU).

The FP32 kernels differentiate the p2g particle math (F_tmp, SVD, von Mises
return map, stress; plb/engine/mpm_simulator.py:122-129, 137-225) in the SVD
basis and evaluate the clamped SVD backward (backward_svd, 137-156, with the
clamp of 184-192) in a cancellation-free form.  These tests restate both the
reference's form and the basis form here and check that they are the same
function: on random particles, elastic and yielding, with singular values
far apart, close together and inside the +-1e-6 clamp.
"""
import numpy as np

DT, MU, LAM, YS = 1e-4, 5e3 / (2 * 1.2), 5e3 * 0.2 / (1.2 * 0.6), 50.0
KS, PM = -1e-4 * (1 / 128) ** 2 * 4 * 64 * 64, (1 / 128) ** 2


def svd_ti(A):
    """SVD with det U = det V = +1 and the sign on the last singular value."""
    U, s, Vt = np.linalg.svd(A)
    V = Vt.T
    if np.linalg.det(U) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    if np.linalg.det(V) < 0:
        V[:, 2] *= -1
        s[2] *= -1
    return U, s, V


def clamp(a):
    return max(a, 1e-6) if a >= 0 else min(a, -1e-6)


def forward(C, F, svd=None):
    Ft = (np.eye(3) + DT * C) @ F
    U, s, V = svd_ti(Ft) if svd is None else svd
    sig = np.maximum(s, 0.05)
    eps = np.log(sig)
    eh = eps - eps.mean()
    nrm = np.sqrt(eh @ eh + 1e-8)
    dg = nrm - YS / (2 * MU)
    y = dg > 0
    e = np.exp(eps - dg / nrm * eh) if y else np.ones(3)
    newF = U @ np.diag(e) @ V.T if y else Ft
    J = np.linalg.det(newF)
    st = 2 * MU * (newF - U @ V.T) @ newF.T + LAM * J * (J - 1) * np.eye(3)
    return KS * st + PM * C, newF, dict(U=U, s=s, V=V, eh=eh, nrm=nrm, dg=dg, y=y, e=e, J=J)


def sigma_grad(P, MN):
    """Gradient of the singular values through the return map (yield branch)."""
    k = P["dg"] / P["nrm"]
    ge2 = np.diag(MN) * P["e"]
    geps = ge2.copy()
    gk = -(ge2 * P["eh"]).sum()
    geh = -k * ge2
    gn = -gk * P["dg"] / P["nrm"] ** 2 + gk / P["nrm"]
    geh = geh + gn * P["eh"] / P["nrm"]
    geps += geh - geh.sum() / 3
    return np.where(P["s"] > 0.05, geps / np.maximum(P["s"], 0.05), 0.0)


def vjp_reference(C, F, P, g_aff, gF1):
    """backward_svd as the reference writes it (U, V gradients, 1/clamp(s_j^2 - s_i^2))."""
    U, s, V, y = P["U"], P["s"], P["V"], P["y"]
    Ft = (np.eye(3) + DT * C) @ F
    newF = U @ np.diag(P["e"]) @ V.T if y else Ft
    A = newF - U @ V.T
    g_raw = KS * g_aff
    tmp = g_raw @ newF
    gR, gN = -2 * MU * tmp, 2 * MU * tmp + gF1
    cof = np.linalg.det(newF) * np.linalg.inv(newF).T
    gN = gN + 2 * MU * g_raw.T @ A + LAM * (2 * P["J"] - 1) * np.trace(g_raw) * cof
    gU, gV, gs = gR @ V, gR.T @ U, np.zeros(3)
    if y:
        gU = gU + gN @ V * P["e"]
        gV = gV + gN.T @ U * P["e"]
        gs = sigma_grad(P, U.T @ gN @ V)
        gFt = np.zeros((3, 3))
    else:
        gFt = gN.copy()
    ss = s ** 2
    Fm = np.array([[0.0 if i == j else 1 / clamp(ss[j] - ss[i]) for j in range(3)] for i in range(3)])
    S = np.diag(s)
    gFt = gFt + U @ ((Fm * (U.T @ gU - gU.T @ U)) @ S) @ V.T + U @ (S @ (Fm * (V.T @ gV - gV.T @ V))) @ V.T \
        + U @ np.diag(gs) @ V.T
    return PM * g_aff + DT * gFt @ F.T, (np.eye(3) + DT * C).T @ gFt


def vjp_basis(C, F, P, g_aff, gF1):
    """The FP32 kernels' form (p2g_particle_vjp_f32 + svd3_bwd_factored_basis)."""
    U, s, V, y = P["U"], P["s"], P["V"], P["y"]
    em1 = P["e"] - 1 if y else s - 1
    ep = 1 + em1
    G = U.T @ (KS * g_aff) @ U
    gJ = LAM * (2 * P["J"] - 1) * np.trace(G)
    MN = U.T @ gF1 @ V
    MR = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            a = 2 * MU * G[i, j] * ep[j]
            MR[i, j] = -a
            MN[i, j] += a + 2 * MU * G[j, i] * em1[j] + (gJ * P["J"] / ep[j] if i == j else 0.0)
    X = np.diag(sigma_grad(P, MN) if y else np.zeros(3))
    k = P["dg"] / P["nrm"] if y else 0.0
    for i, j in ((0, 1), (0, 2), (1, 2)):
        ds, sm = s[j] - s[i], s[j] + s[i]
        f = ds / clamp(ds * sm)
        Kij = MR[i, j] - MR[j, i]
        Kji = -Kij
        if y:
            u = ds / s[i]
            a = 1 - k
            D = P["e"][i] * a / s[i] * (np.expm1(a * np.log1p(u)) / (a * np.log1p(u)) if u != 0 else 1.0) * \
                (np.log1p(u) / u if u != 0 else 1.0)
            se = P["e"][i] + P["e"][j]
            p, m = 0.5 * (D * sm + se), 0.5 * (D * sm - se)
            Kij += MN[i, j] * p + MN[j, i] * m
            Kji += MN[j, i] * p + MN[i, j] * m
        X[i, j], X[j, i] = Kij * f, Kji * f
    Y = X if y else X + MN
    gFt = U @ Y @ V.T
    return PM * g_aff + DT * gFt @ F.T, (np.eye(3) + DT * C).T @ gFt


def _particles(n, seed):
    rng = np.random.default_rng(seed)
    for t in range(n):
        C = rng.normal(size=(3, 3)) * rng.choice([0.5, 5.0])
        if t % 4 == 3:  # two singular values within the clamp: F = Q1 diag(d) Q2
            q1 = np.linalg.qr(rng.normal(size=(3, 3)))[0]
            q2 = np.linalg.qr(rng.normal(size=(3, 3)))[0]
            d = 1 + rng.normal(size=3) * 1e-2
            d[1] = d[0] + 10.0 ** rng.uniform(-9, -6)
            F = q1 @ np.diag(d) @ q2
            C = C * 0
        else:
            F = np.eye(3) + rng.normal(size=(3, 3)) * rng.choice([1e-3, 1e-2, 5e-2])
        yield C, F, rng.normal(size=(3, 3)), rng.normal(size=(3, 3))


def test_basis_form_equals_reference_form():
    worst, kinds = 0.0, set()
    for C, F, g_aff, gF1 in _particles(400, 3):
        _, _, P = forward(C, F)
        kinds.add(bool(P["y"]))
        a = vjp_basis(C, F, P, g_aff, gF1)
        b = vjp_reference(C, F, P, g_aff, gF1)
        for x, r in zip(a, b):
            worst = max(worst, float(np.abs(x - r).max() / np.abs(r).max()))
    assert kinds == {True, False}  # elastic and yielding particles both checked
    assert worst < 1e-9, worst


def test_basis_form_matches_finite_differences_away_from_the_clamp():
    rng = np.random.default_rng(11)
    worst = 0.0
    for C, F, g_aff, gF1 in _particles(120, 5):
        _, _, P = forward(C, F)
        s = P["s"]
        if min(abs(s[i] ** 2 - s[j] ** 2) for i in range(3) for j in range(i + 1, 3)) < 1e-4:
            continue  # the clamped formula is not the derivative there, by design
        if abs(P["dg"]) < 1e-6:
            continue  # the yield test would flip inside the difference step
        gC, gF = vjp_basis(C, F, P, g_aff, gF1)

        def L(C_, F_):
            aff, newF, _ = forward(C_, F_)
            return float((g_aff * aff).sum() + (gF1 * newF).sum())

        h = 1e-7
        fdC, fdF = np.zeros((3, 3)), np.zeros((3, 3))
        for a in range(3):
            for b in range(3):
                E = np.zeros((3, 3))
                E[a, b] = h
                fdC[a, b] = (L(C + E, F) - L(C - E, F)) / (2 * h)
                fdF[a, b] = (L(C, F + E) - L(C, F - E)) / (2 * h)
        worst = max(worst, float(np.abs(gC - fdC).max() / np.abs(fdC).max()),
                    float(np.abs(gF - fdF).max() / np.abs(fdF).max()))
    del rng
    assert worst < 1e-3, worst
