"""Independent numpy restatement of one TTSH3D step, used only to cross-check the C++ oracle.

Unlike the C++ oracle, this follows the reference's storage literally: every
stencil reads from a padded array whose one-cell halo holds the periodic image
(BounPeriU, TTSH3D.cu:1422-1607), and the divergence of u*/P* reads a halo
filled from the previous step's u*/P* (the refresh at the start of getRHS,
TTSH3D.cu:369-371 and :405-407, precedes getVStar, :471-491). Arrays are
indexed [z, y, x]. Only small grids (N <= 16) are meant to be run through it.
"""
import numpy as np


def pad(f, old=None):
    """Pad by one cell; the halo is the periodic image of `old` (default: of f itself)."""
    p = np.pad(f if old is None else old, 1, mode="wrap")
    p[1:-1, 1:-1, 1:-1] = f
    return p


def _sh(fp, dx, dy, dz):
    n = fp.shape[0] - 2
    return fp[1 + dz:1 + dz + n, 1 + dy:1 + dy + n, 1 + dx:1 + dx + n]


def D(fp, a, h):
    """27-point first derivative along axis a (0=x, 1=y, 2=z): d1{x,y,z}CO2I3D, TTSH3D.cu:3280-3328."""
    s = [0, 0, 0]
    acc = 0.0
    w = {0: 16.0 / 36, 1: 4.0 / 36, 2: 1.0 / 36}
    for o1 in (-1, 0, 1):
        for o2 in (-1, 0, 1):
            for sign in (1, -1):
                off = [0, 0, 0]
                off[a] = sign
                others = [b for b in range(3) if b != a]
                off[others[0]] = o1
                off[others[1]] = o2
                acc = acc + sign * w[abs(o1) + abs(o2)] * _sh(fp, *off)
    del s
    return acc / (2.0 * h)


def L(fp, h):
    """15-point Laplacian: laplaceCO2I3D, TTSH3D.cu:3331-3343."""
    corners = sum(_sh(fp, dx, dy, dz) for dx in (-1, 1) for dy in (-1, 1) for dz in (-1, 1))
    faces = sum(_sh(fp, *o) for o in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)])
    return corners / (12 * h * h) + 2.0 / (3 * h * h) * faces - 14.0 / (3 * h * h) * _sh(fp, 0, 0, 0)


def k2_reference(N, h):
    m = np.arange(N)
    k = np.where(m >= N // 2, 2 * np.pi * (m - N) / (N * h), 2 * np.pi * m / (N * h))
    kz, ky, kx = np.meshgrid(k, k, k, indexing="ij")
    k2 = kx * kx + ky * ky + kz * kz
    k2[0, 0, 0] = 1.0
    return k2


def k2_discrete(N, h):
    m = np.arange(N)
    k = np.where(m >= N // 2, 2 * np.pi * (m - N) / (N * h), 2 * np.pi * m / (N * h))
    S = np.sin(k * h) / h
    C = (2 + np.cos(k * h)) / 3
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    Kx = S[x] * C[y] * C[z]
    Ky = C[x] * S[y] * C[z]
    Kz = C[x] * C[y] * S[z]
    return Kx ** 2 + Ky ** 2 + Kz ** 2


def project(Xs, Xold, h, dt, k2_mode, stale):
    N = Xs[0].shape[0]
    pads = [pad(Xs[a], Xold[a] if stale else None) for a in range(3)]
    F = (D(pads[0], 0, h) + D(pads[1], 1, h) + D(pads[2], 2, h)) / dt
    Fh = np.fft.fftn(F)
    if k2_mode == 0:
        Fh = -Fh / k2_reference(N, h)
    else:
        K2 = k2_discrete(N, h)
        Fh = np.where(K2 < 1e-24, 0, -Fh / np.where(K2 < 1e-24, 1, K2))
    return np.fft.ifftn(Fh).real


def step(s, p, k2_mode=0, stale=True):
    """One EEuler step (TTSH3D.cu:347-359) on dict `s` of (N,N,N) arrays; returns a new dict."""
    h, dt = p["h"], p["dt"]
    P = [s["px"], s["py"], s["pz"]]
    V = [s["vx"], s["vy"], s["vz"]]
    phi = s["phi"]
    Pp = [pad(a) for a in P]
    Vp = [pad(a) for a in V]
    phip = pad(phi)
    dP = [[D(Pp[b], a, h) for b in range(3)] for a in range(3)]          # dP[a][b] = D_a P_b
    dphi = [D(phip, a, h) for a in range(3)]
    mu0 = p["aPhi"] * 2 * (phi - 3 * phi * phi + 2 * phi ** 3) - p["kPhi"] * L(phip, h)
    mu = [phi * P[b] + p["La"] ** 2 * L(Pp[b], h) for b in range(3)]
    sig = [[pad(phi * dP[a][b]) for b in range(3)] for a in range(3)]
    P2 = P[0] ** 2 + P[1] ** 2 + P[2] ** 2
    dPhi2 = dphi[0] ** 2 + dphi[1] ** 2 + dphi[2] ** 2
    dtv = []
    for b in range(3):
        r = (-V[0] * D(Vp[b], 0, h) - V[1] * D(Vp[b], 1, h) - V[2] * D(Vp[b], 2, h) + p["mu"] * L(Vp[b], h)
             + mu0 * dphi[b] + p["cA"] * (D(sig[0][b], 0, h) + D(sig[1][b], 1, h) + D(sig[2][b], 2, h)))
        if p.get("zeta", 0.0) != 0.0:
            r = r - p["zeta"] * sum(D(pad(phi * P[a] * P[b]), a, h) for a in range(3))
        dtv.append(r)
    dtp = []
    mup = [pad(m) for m in mu]
    for b in range(3):
        Ab = sum(dphi[a] * dphi[b] * P[a] for a in range(3))
        r = (-V[0] * dP[0][b] - V[1] * dP[1][b] - V[2] * dP[2][b] - p["alpha"] * phi * P[b]
             - p["beta"] * P2 * P[b] + p["eta"] * L(mup[b], h)
             - p["lambda0"] * (P[0] * dP[0][b] + P[1] * dP[1][b] + P[2] * dP[2][b])
             - p["A"] * (dPhi2 * P[b] * P2 + np.sqrt(P2) * Ab))
        dtp.append(r)
    dtphi = -V[0] * dphi[0] - V[1] * dphi[1] - V[2] * dphi[2] + p["gamma"] * L(pad(mu0), h)
    us = [V[b] + dt * dtv[b] for b in range(3)]
    ps = [P[b] + dt * dtp[b] for b in range(3)]
    uold = [s["vxs"], s["vys"], s["vzs"]]
    pold = [s["pxs"], s["pys"], s["pzs"]]
    pv = project(us, uold, h, dt, k2_mode, stale)
    pp = project(ps, pold, h, dt, k2_mode, stale)
    pvp, ppp = pad(pv), pad(pp)
    out = dict(s)
    for b, n in enumerate(("vx", "vy", "vz")):
        out[n] = us[b] - dt * D(pvp, b, h)
        out[n[:2] + "s"] = us[b]
    for b, n in enumerate(("px", "py", "pz")):
        out[n] = ps[b] - dt * D(ppp, b, h)
        out[n[:2] + "s"] = ps[b]
    out["phi"] = phi + dt * dtphi
    out["pv"], out["pp"] = pv, pp
    return out
