"""numpy restatement of the per-snapshot analysis of the reference's readDraw.py and op.py
(test helper): calculate_centroid (readDraw.py:30-52), the centroid z-slice (:222-233) and the
vorticities (:236-237) with op.py's d1xO4 / d1yO4 (op.py:3-13)."""
import numpy as np


def d1xO4(u, h):
    """4th-order periodic derivative along axis 1 (op.py:3-7)."""
    return (np.roll(u, 2, axis=1) - 8 * np.roll(u, 1, axis=1) + 8 * np.roll(u, -1, axis=1)
            - np.roll(u, -2, axis=1)) / (12 * h)


def d1yO4(u, h):
    """4th-order periodic derivative along axis 0 (op.py:9-13)."""
    return (np.roll(u, 2, axis=0) - 8 * np.roll(u, 1, axis=0) + 8 * np.roll(u, -1, axis=0)
            - np.roll(u, -2, axis=0)) / (12 * h)


def centroid(field):
    """readDraw's field is [i][j][k] = (y, x, z); returns the three means (before int())."""
    L = field.shape[0]
    i, j, k = np.meshgrid(np.arange(L), np.arange(L), np.arange(L), indexing="ij")
    m = field.sum()
    return (field * i).sum() / m, (field * j).sum() / m, (field * k).sum() / m


def analyse(phi, P, u, h=1.0):
    """phi, P, u in this repo's [z][y][x] layout; returns the readDraw quantities."""
    to_rd = lambda a: np.transpose(a, (1, 2, 0))  # [z][y][x] -> [y][x][z]
    c = centroid(to_rd(phi))
    idx3 = int(c[2])
    sl = lambda a: to_rd(a)[:, :, idx3]
    vx, vy, vz = sl(u[0]), sl(u[1]), sl(u[2])
    px, py, pz = sl(P[0]), sl(P[1]), sl(P[2])
    return dict(centroid=c, index=tuple(int(x) for x in c), vx=vx, vy=vy, vz=vz, px=px, py=py, pz=pz,
                phi=sl(phi), vortex=d1xO4(vy, h) - d1yO4(vx, h), Pvortex=d1xO4(py, h) - d1yO4(px, h))
