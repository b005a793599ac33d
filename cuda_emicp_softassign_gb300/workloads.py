"""Seeded synthetic point-cloud pairs with the shapes of the benchmark configs.

The reference's demos run on scans that are not redistributed here (the
Stanford bunny in data/bun*.ply) and on pairs made with a random rigid
transform (data/generatePoints.sci). These generators stand in for them. They
are deterministic functions of the seed (numpy PCG64).

Every generator returns ``(X, Y, R_true, t_true)`` with X the target and Y the
source, so that the ideal registration is X ~ R_true Y + t_true.
"""
import numpy as np


def _rot(axis, angle):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)


def random_rotation(rng, max_deg):
    axis = rng.standard_normal(3)
    return _rot(axis, np.radians(rng.uniform(0.0, max_deg)))


def uniform_pair(n=1007, m=None, seed=0, max_deg=30.0, t_range=0.1, noise=1e-3):
    """Config-1 generator: X ~ U[0,1]^3 (n points); Y = R^T (X - t) + N(0, noise^2),
    randomly permuted. For m != n, Y is built from a random subset (m <= n) or
    from extra uniform points (m > n)."""
    rng = np.random.default_rng(seed)
    m = n if m is None else m
    base = rng.uniform(0.0, 1.0, (max(n, m), 3))
    X = base[:n]
    R = random_rotation(rng, max_deg)
    t = rng.uniform(-t_range, t_range, 3)
    idx = rng.permutation(max(n, m))[:m]
    src = base[idx]
    Y = (src - t) @ R + rng.normal(0.0, noise, (m, 3))  # R^T (x - t) for row vectors
    return X.astype(np.float32), Y.astype(np.float32), R, t


def _ellipsoid_surface(rng, n, count=3):
    """n points on a union of `count` random ellipsoids (semi-axes U[0.02, 0.08]),
    with outward normals."""
    centres = rng.uniform(-0.05, 0.05, (count, 3))
    axes = rng.uniform(0.02, 0.08, (count, 3))
    rots = [random_rotation(rng, 180.0) for _ in range(count)]
    pts, nrm = [], []
    per = np.full(count, n // count)
    per[: n - per.sum()] += 1
    for k in range(count):
        u = rng.standard_normal((per[k], 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        p = u * axes[k]
        g = u / axes[k]  # gradient of the implicit function
        g /= np.linalg.norm(g, axis=1, keepdims=True)
        pts.append(p @ rots[k].T + centres[k])
        nrm.append(g @ rots[k].T)
    return np.concatenate(pts), np.concatenate(nrm)


def _view(rng, P, Nrm, keep_frac=0.7):
    """Keeps the keep_frac of points whose normal best faces a random direction."""
    v = rng.standard_normal(3)
    v /= np.linalg.norm(v)
    score = Nrm @ v
    k = int(round(keep_frac * len(P)))
    idx = np.argsort(-score)[:k]
    return P[idx]


def surface_pair(n=2000, m=None, seed=0, n_surface=40000, surface_noise=5e-4, rot_deg_y=45.0,
                 max_deg=None, t_range=0.02, outlier_frac=0.0):
    """Config-2/3/5 generator: two ~70% views of a union of 3 ellipsoids.

    The second view is transformed by G (45 deg about y, or a random rotation
    of up to max_deg, plus t ~ U[-t_range, t_range]^3) and becomes Y. Each
    view is randomly subsampled to n (X) / m (Y) points; outlier_frac of
    each view is replaced by uniform points in the bounding box."""
    rng = np.random.default_rng(seed)
    m = n if m is None else m
    need = max(n, m) / 0.7 * 1.05
    n_surface = int(max(n_surface, need))
    P, Nrm = _ellipsoid_surface(rng, n_surface)
    P = P + rng.normal(0.0, surface_noise, P.shape)
    v1 = _view(rng, P, Nrm)
    v2 = _view(rng, P, Nrm)

    def sub(v, k):
        k_out = int(round(outlier_frac * k))
        k_in = k - k_out
        idx = rng.choice(len(v), size=k_in, replace=len(v) < k_in)
        pts = v[idx]
        if k_out:
            lo, hi = P.min(0), P.max(0)
            pts = np.concatenate([pts, rng.uniform(lo, hi, (k_out, 3))])
            pts = pts[rng.permutation(k)]
        return pts

    X = sub(v1, n)
    Y0 = sub(v2, m)
    if max_deg is None:
        G = _rot([0.0, 1.0, 0.0], np.radians(rot_deg_y))
    else:
        G = random_rotation(rng, max_deg)
    g = rng.uniform(-t_range, t_range, 3)
    Y = Y0 @ G.T + g
    # X ~ G^T (Y - g)  =>  R_true = G^T, t_true = -G^T g
    return X.astype(np.float32), Y.astype(np.float32), G.T, -G.T @ g


# Named configurations (the benchmark configs). Sizes are the full sizes.
CONFIGS = {
    "c1_emicp_1007": dict(kind="emicp", gen="uniform", n=1007),
    "c2_softassign_2000": dict(kind="softassign", gen="surface", n=2000),
    "c3_emicp_40097": dict(kind="emicp", gen="surface", n=40097, max_deg=20.0, outlier_frac=0.05),
    "c5_softassign_20000": dict(kind="softassign", gen="surface", n=20000),
    # ICP on config 3's clouds (no benchmark config of the reference names ICP)
    "icp_40097": dict(kind="icp", gen="surface", n=40097, max_deg=20.0, outlier_frac=0.05),
}


def make(config, seed=0, n=None):
    """Point pair for a named config (optionally at a smaller size n)."""
    c = dict(CONFIGS[config])
    size = n or c.pop("n")
    c.pop("n", None)
    kind = c.pop("kind")
    gen = c.pop("gen")
    if gen == "uniform":
        X, Y, R, t = uniform_pair(n=size, seed=seed, **c)
    else:
        X, Y, R, t = surface_pair(n=size, seed=seed, **c)
    return kind, X, Y, R, t


def batch_pairs(count=256, seed=0, lo=500, hi=20000):
    """Config-4 generator: `count` pairs, N and M log-uniform in [lo, hi], the
    config-1 generator per pair (own seed); even indices EM-ICP, odd Softassign."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        m = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        X, Y, R, t = uniform_pair(n=n, m=m, seed=int(rng.integers(1 << 31)))
        out.append(("emicp" if k % 2 == 0 else "softassign", X, Y, R, t))
    return out


def rotation_error_deg(A, B):
    """Angle of A B^T in degrees, robust for tiny angles."""
    M = np.asarray(A, dtype=np.float64) @ np.asarray(B, dtype=np.float64).T
    s = np.linalg.norm([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]]) / 2.0
    c = (np.trace(M) - 1.0) / 2.0
    return float(np.degrees(np.arctan2(s, c)))
