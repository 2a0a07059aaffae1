"""Oracle restatement of the single-vector LOBPCG in ``rqutils/ground_locg.py``.

Test infrastructure only.  The operation order follows the reference so that iteration counts
reproduce: iteration 0 (264-272), iteration 1 with a 2x2 Rayleigh-Ritz (274-286), then the loop
body (288-341) with the double-pass projection (380-421), three-vector Rayleigh-Ritz (235-255),
Cardano eigenpair (438-471) and the self-consistency convergence test (329-334).
"""
import numpy as np


def _vdot(a, b):
    """sum(conj(a) * b) -- the reference's reduction form (ground_locg.py:214, 243)."""
    return np.sum(np.conjugate(a) * b)


def _norm(a):
    return np.linalg.norm(a)


def eigenpair_2x2(m):
    """Lowest eigenpair of a Hermitian 2x2 (ground_locg.py:424-435)."""
    d0, d1 = np.real(m[0, 0]), np.real(m[1, 1])
    off = m[1, 0]
    det = d0 * d1 - np.abs(off) ** 2
    tr = d0 + d1
    lam = (tr - np.sqrt(tr * tr - 4. * det)) * 0.5
    v = np.array([(d1 - lam + np.conjugate(off)) / (d0 - lam + off), -1.])
    v = v / np.sqrt(np.real(v[0]) ** 2 + np.imag(v[0]) ** 2 + 1.)
    return lam, v


def eigenpair_3x3(m):
    """Lowest eigenpair of a Hermitian 3x3 by Cardano's formula (J. Kopp, Int. J. Mod. Phys. C 19,
    523 (2008)), as ground_locg.py:438-471: characteristic polynomial coefficients c2, c1, c0, the
    trigonometric root with the smallest value, and the eigenvector as the conjugated cross product
    of columns 1 and 2 of (A - lambda I)."""
    d = np.real(np.diagonal(m))
    mod10, mod20, mod21 = np.abs(m[1, 0]) ** 2, np.abs(m[2, 0]) ** 2, np.abs(m[2, 1]) ** 2
    c2 = -(d[0] + d[1] + d[2])
    c1 = (d[0] * d[2] + d[1] * d[0] + d[2] * d[1]) - (mod10 + mod20 + mod21)
    c0 = d[0] * mod21 + d[1] * mod20 + d[2] * mod10
    c0 -= d[0] * d[1] * d[2]
    c0 -= 2. * np.real(m[0, 2] * m[1, 0] * m[2, 1])
    p = c2 * c2 - 3. * c1
    q = -13.5 * c0 - c2 * c2 * c2 + 4.5 * c2 * c1
    with np.errstate(invalid='ignore'):
        phi = np.arctan2(np.sqrt(27. * (0.25 * c1 * c1 * (p - c1) + c0 * (q + 6.75 * c0))), q) / 3.
        cphi, sphi = np.cos(phi), np.sin(phi)
        s3 = np.sqrt(3.)
        xmin = min(2. * cphi, -cphi - s3 * sphi, -cphi + s3 * sphi)
        lam = np.sqrt(p) / 3. * xmin - c2 / 3.
    col1 = np.array(m[:, 1], copy=True)
    col1[1] -= lam
    col2 = np.array(m[:, 2], copy=True)
    col2[2] -= lam
    v = np.conjugate(np.cross(col1, col2))
    v = v / np.sqrt(np.sum(np.real(v) ** 2 + np.imag(v) ** 2))
    return lam, v


def project_out(basis, vec):
    """_project_out, ground_locg.py:380-421: two classical Gram-Schmidt passes with
    normalisation, two without, then zero the result if its norm is below 0.99."""
    v = vec
    for _ in range(2):
        ips = [_vdot(b, v) for b in basis]
        for b, ip in zip(basis, ips):
            v = v - b * ip
        nv = _norm(v)
        v = v / (1. if nv == 0. else nv)
    for _ in range(2):
        ips = [_vdot(b, v) for b in basis]
        for b, ip in zip(basis, ips):
            v = v - b * ip
    return v * (1. if _norm(v) >= 0.99 else 0.)


def rayleigh_ritz(matvec, vectors, counter):
    """compute_sas + eigenpair, ground_locg.py:235-255.  Strict lower triangle from w_b^H A w_a,
    mirrored by conjugate transpose, diagonal w_a^H A w_a.  One matvec per vector."""
    nv = len(vectors)
    sas = np.zeros((nv, nv), dtype=vectors[0].dtype)
    mvs = []
    for a, va in enumerate(vectors):
        mva = matvec(va)
        counter[0] += 1
        mvs.append(mva)
        for b in range(a + 1, nv):
            sas[b, a] = _vdot(vectors[b], mva)
    sas = sas + np.conjugate(sas).T
    for a, (va, mva) in enumerate(zip(vectors, mvs)):
        sas[a, a] = _vdot(va, mva)
    return eigenpair_2x2(sas) if nv == 2 else eigenpair_3x3(sas)


def ground_locg(matvec, xinit, maxiter=1000, tol=None, tol_dim=None, vspace=None, history=None):
    """_ground_locg_callable, ground_locg.py:182-377 (debug=False path).

    ``xinit`` may be an integer index (one-hot, needs ``vspace=(dim, dtype)``, 201-206).
    ``tol`` defaults to the dtype's machine epsilon (208-209).  ``tol_dim`` is the vector length
    used in the convergence test (330); the reference uses its padded ``states_size`` there.
    ``history`` (a list) receives (theta, |r|) per loop iteration.  Returns (theta, x, niter)."""
    if np.issubdtype(np.asarray(xinit).dtype, np.integer):
        dim, dtype = vspace
        x0 = np.zeros(dim, dtype=dtype)
        x0[int(xinit)] = 1
        xinit = x0
    xinit = np.asarray(xinit)
    if tol is None:
        tol = float(np.finfo(xinit.dtype).eps)
    if tol_dim is None:
        tol_dim = xinit.shape[0]
    counter = [0]

    def mv(v):
        counter[0] += 1
        return matvec(v)

    x = xinit / _norm(xinit)
    # iteration 0 (264-272)
    ax = mv(x)
    rho = np.real(_vdot(x, ax))
    r = ax - rho * x
    # iteration 1 (274-286)
    nr = _norm(r)
    p = r / (1. if nr == 0. else nr)
    theta, kappa = rayleigh_ritz(matvec, (x, p), counter)
    t = p * kappa[0] - x * kappa[1]
    u = x * kappa[0] + p * kappa[1]
    x = u / _norm(u)
    y = t / _norm(t)
    r = mv(x) - theta * x
    # loop (288-341, 366-370)
    niter, converged, theta = 0, False, 0.
    while niter < maxiter and not converged:
        p = project_out((x, y), r)
        theta, kappa = rayleigh_ritz(matvec, (x, y, p), counter)
        s = y * kappa[1] + p * kappa[2]
        ns = _norm(s)
        t = s * (kappa[0] / ns) - x * ns
        u = x * kappa[0] + s
        xn = u / _norm(u)
        yn = t / _norm(t)
        axn = mv(xn)
        r = axn - xn * theta
        reltol = (_norm(axn) - theta) * tol_dim * 10
        nr = _norm(r)
        converged = bool(nr < tol * reltol)
        if history is not None:
            history.append((float(np.real(theta)), float(nr)))
        x, y = xn, yn
        niter += 1
    ground_locg.last_matvecs = counter[0]
    return theta, x, niter
