"""NumPy restatement of the neural radiance cache's network, for the GPU tests.

Mirrors radiancecascade_gb300/csrc/rc_nrc.cuh: the multiresolution hash
encoding of (probe centre, direction texel, cascade) (FP16 table, one cell per
level), the 16 direction/cascade features, and the MLP with BF16 weights and activations and wide (here FP64)
accumulation, forward and backward.  Test infrastructure only.
"""
import numpy as np

HASH_LEVELS = 16
PARAMS = 4 * (64 * 64 + 64) + 16 * 64 + 16


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack_save(blob, hash_log2):
    """rc_nrc_save's layout: an 88-byte header (with rc_nrc_params), the MLP (FP32), the hash grid (FP32)."""
    head = 4 * 4 + 8 + 64  # magic, version, mlp_count, pad, hash_count, rc_nrc_params (64 bytes)
    mlp = np.frombuffer(blob, np.float32, PARAMS, head)
    n_hash = HASH_LEVELS * (1 << hash_log2) * 2
    table = np.frombuffer(blob, np.float32, n_hash, head + PARAMS * 4)
    return mlp.copy(), table.reshape(HASH_LEVELS, 1 << hash_log2, 2).copy()


def layers(mlp):
    W, b = [], []
    for l in range(4):
        o = l * (64 * 64 + 64)
        W.append(mlp[o:o + 4096].reshape(64, 64))
        b.append(mlp[o + 4096:o + 4160])
    o = 4 * (64 * 64 + 64)
    W.append(mlp[o:o + 1024].reshape(16, 64))
    b.append(mlp[o + 1024:o + 1040])
    return W, b


def resolutions(base, top):
    g = np.exp((np.log(top) - np.log(base)) / (HASH_LEVELS - 1))
    return [max(1, int(np.floor(base * g ** l + 1e-9))) for l in range(HASH_LEVELS)]


def dir_resolutions():
    return [max(1, int(np.floor(2.0 * 64.0 ** (l / (HASH_LEVELS - 1)) + 1e-9))) for l in range(HASH_LEVELS)]


def encode(table16, res, dres, log2T, probe_xyz, spacing, extent, dirs, n, cascade):
    """Hash features (32) of queries: probes at lattice indices probe_xyz [q, 3],
    direction texels dirs [q] of an n x n octahedral map, cascade index."""
    T = 1 << log2T
    inv = np.float32(1.0) / np.float32(extent)
    u = ((probe_xyz.astype(np.float32) * np.float32(spacing) + np.float32(0.5 * spacing)) * inv).astype(np.float32)
    du = ((dirs % n).astype(np.float32) + np.float32(0.5)) / np.float32(n)
    dv = ((dirs // n).astype(np.float32) + np.float32(0.5)) / np.float32(n)
    out = np.zeros((len(u), 32), np.float32)
    m32 = 0xFFFFFFFF
    for l, (r, q) in enumerate(zip(res, dres)):
        c = [np.minimum((u[:, a] * np.float32(r)).astype(np.int64), r - 1).astype(np.uint64) for a in range(3)]
        a_ = np.minimum((du * np.float32(q)).astype(np.int64), q - 1).astype(np.uint64)
        b_ = np.minimum((dv * np.float32(q)).astype(np.int64), q - 1).astype(np.uint64)
        h = (c[0] ^ ((c[1] * 2654435761) & m32) ^ ((c[2] * 805459861) & m32) ^ ((a_ * 0x85EBCA77) & m32)
             ^ ((b_ * 0xC2B2AE3D) & m32) ^ ((cascade * 0x27D4EB2F) & m32))
        out[:, 2 * l:2 * l + 2] = table16[l, (h & (T - 1)).astype(np.int64)].astype(np.float32)
    return out


def dir_features(n, dirs, level_slot):
    tx, ty = dirs % n, dirs // n
    u = (2.0 * tx + 1.0) / n - 1.0
    v = (2.0 * ty + 1.0) / n - 1.0
    f = np.stack([u, v, np.sin(np.pi * u), np.cos(np.pi * u), np.sin(np.pi * v), np.cos(np.pi * v),
                  np.sin(2 * np.pi * u), np.cos(2 * np.pi * u), np.sin(2 * np.pi * v), np.cos(2 * np.pi * v)], 1)
    onehot = np.zeros((len(dirs), 6))
    onehot[:, min(level_slot, 5)] = 1.0
    return bf16(np.concatenate([f, onehot], 1).astype(np.float32))


def forward(W, b, x):
    """x [n, 64] (float32) -> outputs [n, 16] and the saved activations."""
    acts = [bf16(x)]
    h = acts[0]
    for l in range(4):
        z = h.astype(np.float64) @ bf16(W[l]).astype(np.float64).T + b[l]
        h = bf16(np.maximum(z, 0.0).astype(np.float32))
        acts.append(h)
    o = h.astype(np.float64) @ bf16(W[4]).astype(np.float64).T + b[4]
    return o, acts


def served(o, scale):
    """T = [o_3 >= 1/2]; R = 0 where T = 1, else max(o / scale, 0)."""
    t = (o[:, 3:4] >= 0.5).astype(np.float64)
    return np.concatenate([np.where(t > 0, 0.0, np.maximum(o[:, :3] / scale, 0.0)), t], 1)


def backward(W, b, x, y, scale):
    """Gradient of sum((o - y')^2) / n, y' = (R * scale, T); -> (param grad, position grad [32])."""
    n = len(x)
    o, acts = forward(W, b, x)
    yy = np.concatenate([y[:, :3] * scale, y[:, 3:4]], 1)
    e = np.zeros((n, 16))
    e[:, :4] = 2.0 * (o[:, :4] - yy) / n
    e = e.astype(np.float32).astype(np.float64)
    g = np.zeros(PARAMS)
    o4 = 4 * (64 * 64 + 64)
    g[o4:o4 + 1024] = (e.T @ acts[4].astype(np.float64)).ravel()
    g[o4 + 1024:o4 + 1040] = e.sum(0)
    dx = bf16(e.astype(np.float32)).astype(np.float64) @ bf16(W[4]).astype(np.float64)
    for l in range(3, -1, -1):
        dz = bf16((dx * (acts[l + 1] > 0)).astype(np.float32)).astype(np.float64)
        o0 = l * (64 * 64 + 64)
        g[o0:o0 + 4096] = (dz.T @ acts[l].astype(np.float64)).ravel()
        g[o0 + 4096:o0 + 4160] = dz.sum(0)
        dx = dz @ bf16(W[l]).astype(np.float64)
    return g, dx[:, :32].sum(0)
