"""Seeded synthetic inputs for the spatial-query workloads.

The reference publishes no dataset for this path; every workload is generated here from a recorded 64-bit seed with the
shapes, sizes and value distributions of the benchmark configurations:

* ``noisy_icosphere``: the icosahedron refined by repeated 4-to-1 edge-midpoint subdivision with midpoints pushed to the
  unit sphere (the rule of GeodesicSphere3::compute, Code/Source/Algorithms/GeodesicSphere3.cpp:28-134), then each vertex
  displaced radially by N(0, sigma). Six subdivisions give 81,920 triangles and 40,962 vertices.
* ``heightfield``: an n x n vertex grid over [0,1]^2 with z from seeded value-noise fBm, two triangles per cell.
* uniform query boxes, plane-origin cosine-distributed rays, and the batched/serving mixtures.

Vertex order is this generator's own; only the mesh, not its numbering, is specified by the workloads.
"""

import numpy as np

# Regular icosahedron (unit circumradius): the classic coordinates a = 0.5257..., b = 0.8506...
_ICO_A = 0.525731112119133606
_ICO_B = 0.850650808352039932
_ICO_V = np.array([
    [-_ICO_A, 0.0, _ICO_B], [_ICO_A, 0.0, _ICO_B], [-_ICO_A, 0.0, -_ICO_B], [_ICO_A, 0.0, -_ICO_B],
    [0.0, _ICO_B, _ICO_A], [0.0, _ICO_B, -_ICO_A], [0.0, -_ICO_B, _ICO_A], [0.0, -_ICO_B, -_ICO_A],
    [_ICO_B, _ICO_A, 0.0], [-_ICO_B, _ICO_A, 0.0], [_ICO_B, -_ICO_A, 0.0], [-_ICO_B, -_ICO_A, 0.0]], np.float64)
_ICO_F = np.array([
    [1, 4, 0], [4, 9, 0], [4, 5, 9], [8, 5, 4], [1, 8, 4], [1, 10, 8], [10, 3, 8], [8, 3, 5], [3, 2, 5], [3, 7, 2],
    [3, 10, 7], [10, 6, 7], [6, 11, 7], [6, 0, 11], [6, 1, 0], [10, 1, 6], [11, 0, 9], [2, 11, 9], [5, 2, 9],
    [11, 2, 7]], np.int64)

CONFIG_SEEDS = {0: 0x7E4A0000, 1: 0x7E4A0001, 2: 0x7E4A0002, 3: 0x7E4A0003, 4: 0x7E4A0004}

_SPHERE_CACHE = {}


def icosphere(subdivisions):
    """Unit geodesic sphere: float64 vertices (V, 3) and int64 faces (F, 3)."""
    if subdivisions in _SPHERE_CACHE:
        return _SPHERE_CACHE[subdivisions]
    V = _ICO_V.copy()
    F = _ICO_F.copy()
    for _ in range(subdivisions):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (len(V) + 1) + e[:, 1]
        ukey, inv = np.unique(key, return_inverse=True)
        a = ukey // (len(V) + 1)
        b = ukey % (len(V) + 1)
        mid = V[a] + V[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(V)
        V = np.concatenate([V, mid])
        nf = len(F)
        m01 = base + inv[:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:]
        F = np.concatenate([
            np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
            np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    _SPHERE_CACHE[subdivisions] = (V, F)
    return V, F


def noisy_icosphere(subdivisions, seed, sigma=0.01, radius=1.0, scale=None, center=None):
    """Icosphere with radial N(0, sigma) vertex noise and an optional per-axis stretch; float32 V, int32 F."""
    V, F = icosphere(subdivisions)
    rng = np.random.default_rng(seed)
    r = radius + rng.normal(0.0, sigma, size=len(V))
    P = V * r[:, None]
    if scale is not None:
        P = P * np.asarray(scale, np.float64)[None, :]
    if center is not None:
        P = P + np.asarray(center, np.float64)[None, :]
    return P.astype(np.float32), F.astype(np.int32)


def uniform_box_points(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    return (lo + (hi - lo) * rng.random((n, 3))).astype(np.float32)


def _value_noise(x, y, freq, rng):
    """Value noise on a (freq+1)^2 lattice of uniform values, smoothstep-interpolated, periodic-free."""
    lat = rng.random((freq + 1, freq + 1))
    fx = x * freq
    fy = y * freq
    ix = np.minimum(np.floor(fx).astype(np.int64), freq - 1)
    iy = np.minimum(np.floor(fy).astype(np.int64), freq - 1)
    tx = fx - ix
    ty = fy - iy
    sx = tx * tx * (3.0 - 2.0 * tx)
    sy = ty * ty * (3.0 - 2.0 * ty)
    v00 = lat[ix, iy]
    v10 = lat[ix + 1, iy]
    v01 = lat[ix, iy + 1]
    v11 = lat[ix + 1, iy + 1]
    a = v00 + (v10 - v00) * sx
    b = v01 + (v11 - v01) * sx
    return (a + (b - a) * sy) * 2.0 - 1.0


def heightfield(n, seed, octaves=6, amplitude=0.1, lacunarity=2.0, gain=0.5, base_freq=4):
    """n x n vertex grid over [0,1]^2 (2 (n-1)^2 triangles) with fBm value-noise heights; float32 V, int32 F."""
    rng = np.random.default_rng(seed)
    u = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(u, u, indexing="ij")
    Z = np.zeros_like(X)
    amp = amplitude
    freq = float(base_freq)
    for _ in range(octaves):
        Z += amp * _value_noise(X, Y, int(round(freq)), rng)
        amp *= gain
        freq *= lacunarity
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(np.float32)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i, indexing="ij")
    v00 = (I * n + J).ravel()
    v10 = ((I + 1) * n + J).ravel()
    v01 = (I * n + J + 1).ravel()
    v11 = ((I + 1) * n + J + 1).ravel()
    F = np.empty((2 * len(v00), 3), np.int64)
    F[0::2] = np.stack([v00, v10, v11], 1)
    F[1::2] = np.stack([v00, v11, v01], 1)
    return V, F.astype(np.int32)


def cosine_rays_down(n, seed, z0=0.5):
    """Origins uniform on the plane z = z0 over [0,1]^2; unit directions cosine-distributed about -z."""
    rng = np.random.default_rng(seed)
    o = np.empty((n, 3), np.float64)
    o[:, :2] = rng.random((n, 2))
    o[:, 2] = z0
    u1 = rng.random(n)
    u2 = rng.random(n)
    r = np.sqrt(u1)
    phi = 2.0 * np.pi * u2
    d = np.stack([r * np.cos(phi), r * np.sin(phi), -np.sqrt(np.maximum(0.0, 1.0 - u1))], 1)
    return o.astype(np.float32), d.astype(np.float32)


def random_rays(n, lo, hi, seed):
    """Origins uniform in a box, directions uniform on the sphere (not normalised to any particular length)."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    o = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


# ---------------------------------------------------------------------------------------------------------------------
# Benchmark configurations (full sizes) and reduced parity sizes
# ---------------------------------------------------------------------------------------------------------------------

def config0(scale=1.0):
    """Plain closest point: icosphere subdiv 6 (81,920 tris), 262,144 queries in [-1.5,1.5]^3."""
    s = CONFIG_SEEDS[0]
    sub = 6 if scale >= 1.0 else max(2, int(round(6 + np.log(scale) / np.log(4))))
    V, F = noisy_icosphere(sub, s)
    nq = int(262144 * scale) if scale < 1.0 else 262144
    Q = uniform_box_points(max(nq, 1), [-1.5] * 3, [1.5] * 3, s + 1)
    return V, F, Q


def config3_spec(num_meshes=4096, seed=CONFIG_SEEDS[3], min_level=2, max_level=7, min_q=1000, max_q=100000):
    """Per-mesh parameters of the batched workload: subdivision level (uniform over min..max, so triangle counts are
    log-uniform from 20 * 4^min to 20 * 4^max), per-axis stretch U[0.5, 2], log-uniform query count, noise seed."""
    rng = np.random.default_rng(seed)
    levels = rng.integers(min_level, max_level + 1, size=num_meshes)
    scales = rng.uniform(0.5, 2.0, size=(num_meshes, 3))
    nq = np.exp(rng.uniform(np.log(min_q), np.log(max_q), size=num_meshes)).astype(np.int64)
    mesh_seeds = rng.integers(0, 2 ** 31 - 1, size=num_meshes)
    return levels, scales, nq, mesh_seeds


def config3_numpy(num_meshes, seed=CONFIG_SEEDS[3], **kw):
    """Concatenated batch (host arrays): V, F (indices into V), face_offsets, queries, query_offsets, levels.
    Each mesh is a seeded noisy icosphere with an affine stretch; its queries are uniform in its box grown by 50%."""
    levels, scales, nq, seeds = config3_spec(num_meshes, seed, **kw)
    Vs, Fs, Qs = [], [], []
    vbase = 0
    for m in range(num_meshes):
        V, F = noisy_icosphere(int(levels[m]), int(seeds[m]), scale=scales[m])
        lo, hi = V.min(0).astype(np.float64), V.max(0).astype(np.float64)
        c, e = 0.5 * (lo + hi), 1.5 * (hi - lo)
        Q = uniform_box_points(int(nq[m]), c - 0.5 * e, c + 0.5 * e, int(seeds[m]) + 1)
        Vs.append(V)
        Fs.append(F + vbase)
        Qs.append(Q)
        vbase += len(V)
    face_off = np.concatenate([[0], np.cumsum([len(f) for f in Fs])]).astype(np.int64)
    q_off = np.concatenate([[0], np.cumsum([len(q) for q in Qs])]).astype(np.int64)
    return (np.concatenate(Vs), np.concatenate(Fs).astype(np.int32), face_off, np.concatenate(Qs), q_off, levels)


def config3_torch(num_meshes=4096, seed=CONFIG_SEEDS[3], device="cuda", **kw):
    """The batched workload generated on the GPU (same per-mesh parameters as config3_numpy; noise and queries drawn
    with torch's generator, so values differ from the NumPy version). Returns CUDA tensors V, F, query positions and
    query offsets, plus host face offsets (int64) and per-mesh levels."""
    import torch
    levels, scales, nq, seeds = config3_spec(num_meshes, seed, **kw)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    nv_l = {L: len(icosphere(L)[0]) for L in range(int(levels.min()), int(levels.max()) + 1)}
    nf_l = {L: len(icosphere(L)[1]) for L in nv_l}
    nv = np.array([nv_l[int(L)] for L in levels], np.int64)
    nf = np.array([nf_l[int(L)] for L in levels], np.int64)
    voff = np.concatenate([[0], np.cumsum(nv)])
    foff = np.concatenate([[0], np.cumsum(nf)]).astype(np.int64)
    qoff = np.concatenate([[0], np.cumsum(nq)]).astype(np.int64)
    V = torch.empty((int(voff[-1]), 3), dtype=torch.float32, device=device)
    F = torch.empty((int(foff[-1]), 3), dtype=torch.int32, device=device)
    sc = torch.as_tensor(scales, dtype=torch.float32, device=device)
    for L in nv_l:
        ms = np.nonzero(levels == L)[0]
        if len(ms) == 0:
            continue
        tv, tf = icosphere(L)
        tv = torch.as_tensor(tv, dtype=torch.float32, device=device)
        tf = torch.as_tensor(tf, dtype=torch.int64, device=device)
        msd = torch.as_tensor(ms, device=device)
        r = 1.0 + 0.01 * torch.randn((len(ms), len(tv), 1), generator=g, device=device)
        vals = tv[None] * r * sc[msd][:, None, :]
        vb = torch.as_tensor(voff[ms], device=device)
        V[(vb[:, None] + torch.arange(len(tv), device=device)[None]).reshape(-1)] = vals.reshape(-1, 3)
        fb = torch.as_tensor(foff[ms], device=device)
        F[(fb[:, None] + torch.arange(len(tf), device=device)[None]).reshape(-1)] = \
            (tf[None] + vb[:, None, None]).reshape(-1, 3).to(torch.int32)
    mesh_of_v = torch.repeat_interleave(torch.arange(num_meshes, device=device), torch.as_tensor(nv, device=device))
    lo = torch.full((num_meshes, 3), float("inf"), device=device).scatter_reduce(
        0, mesh_of_v[:, None].expand(-1, 3), V, reduce="amin")
    hi = torch.full((num_meshes, 3), float("-inf"), device=device).scatter_reduce(
        0, mesh_of_v[:, None].expand(-1, 3), V, reduce="amax")
    c, e = 0.5 * (lo + hi), 1.5 * (hi - lo)
    mesh_of_q = torch.repeat_interleave(torch.arange(num_meshes, device=device), torch.as_tensor(nq, device=device))
    u = torch.rand((int(qoff[-1]), 3), generator=g, device=device)
    Q = (c[mesh_of_q] + (u - 0.5) * e[mesh_of_q]).contiguous()
    qoff_d = torch.as_tensor(qoff, device=device)
    return V, F, foff, Q, qoff_d, levels


def config1(grid=1024, nrays=4194304):
    """Ray first hit: 1024^2 heightfield (2,093,058 tris), 4,194,304 cosine rays from z = 0.5."""
    s = CONFIG_SEEDS[1]
    V, F = heightfield(grid, s)
    o, d = cosine_rays_down(nrays, s + 1)
    return V, F, o, d
