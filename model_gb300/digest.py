"""Size-independent digests of 3-D fields, for comparing long runs.

A digest of an N-point field x holds:
  proj   m random projections r_i . x with r_i in {-1, +1}^N (splitmix64
         signs, so identical on every platform).  For two fields a and b,
         |P a - P b| / sqrt(m) is an unbiased estimate of |a - b| (its square
         has relative variance 2/m), so the relative L2 error of a whole field
         can be checked against a digest of a few hundred bytes;
  norm   the L2 norm of x;
  level  the L2 norm of every level k (x viewed as [i][j][k]);
  idx    seeded sample positions, and
  sample the values of x there.

Digests let a run of a few hundred steps on a 16.7 M-point grid be pinned by a
fixture of kilobytes instead of the end state itself.
"""
from __future__ import annotations

import numpy as np

from model_gb300.configs import splitmix_uniform

PROJ_SEED = 0x5EED0000
SAMPLE_SEED = 0x5A3F0000
CHUNK = 1 << 22


def _stream(seed: int, start: int, n: int) -> np.ndarray:
    # splitmix_uniform(seed, n) draws elements 1..n of the stream; element j of
    # stream `seed` equals element j - start of stream seed + start * gamma, so
    # a chunk that starts at `start` is the stream of that shifted seed
    gamma = 0x9E3779B97F4A7C15
    return splitmix_uniform((seed + start * gamma) & 0xFFFFFFFFFFFFFFFF, n)


def projections(fields: list, m: int, seed: int = PROJ_SEED) -> np.ndarray:
    """[len(fields), m] projections of equally long fields."""
    n = fields[0].size
    flat = [np.ascontiguousarray(f, dtype=np.float64).ravel() for f in fields]
    out = np.zeros((len(flat), m))
    for r in range(m):
        s = seed + (r << 40)
        for c0 in range(0, n, CHUNK):
            c = min(CHUNK, n - c0)
            sg = _stream(s, c0, c)
            sg = np.where(sg < 0.5, -1.0, 1.0)
            for f, x in enumerate(flat):
                out[f, r] += float(np.dot(sg, x[c0:c0 + c]))
    return out


def sample_positions(n: int, count: int, seed: int = SAMPLE_SEED) -> np.ndarray:
    count = min(count, n)
    u = splitmix_uniform(seed, count)
    return np.minimum((u * n).astype(np.int64), n - 1)


def digest(fields: dict, shape: tuple, m: int = 64, samples: int = 8192) -> dict:
    """Digest of every field of `fields` (name -> array of `shape`)."""
    names = sorted(fields)
    arrs = [np.asarray(fields[k], dtype=np.float64).reshape(shape) for k in names]
    n = arrs[0].size
    idx = sample_positions(n, samples)
    proj = projections(arrs, m)
    out = {"digest_m": np.int64(m), "digest_idx": idx}
    for f, (k, a) in enumerate(zip(names, arrs)):
        flat = a.ravel()
        out[f"proj_{k}"] = proj[f]
        out[f"norm_{k}"] = np.float64(np.linalg.norm(flat))
        out[f"level_{k}"] = np.sqrt(np.sum(a * a, axis=(0, 1)))
        out[f"sample_{k}"] = flat[idx]
    return out


def compare(fields: dict, ref: dict) -> dict:
    """Relative errors of `fields` against the digest `ref`, per field:
    proj (the projection estimate of the whole field's relative L2 error),
    sample (relative L2 over the sampled points), level (largest relative
    error of a level norm) and norm."""
    m = int(ref["digest_m"])
    idx = ref["digest_idx"]
    names = sorted(fields)
    arrs = [np.asarray(fields[k], dtype=np.float64) for k in names]
    proj = projections(arrs, m)
    out = {}
    for f, (k, a) in enumerate(zip(names, arrs)):
        nref = float(ref[f"norm_{k}"])
        scale = nref if nref > 0 else 1.0
        flat = a.ravel()
        e_proj = float(np.linalg.norm(proj[f] - ref[f"proj_{k}"]) / np.sqrt(m)) / scale
        sr = ref[f"sample_{k}"]
        ns = float(np.linalg.norm(sr))
        e_samp = float(np.linalg.norm(flat[idx] - sr)) / (ns if ns > 0 else 1.0)
        lv = np.sqrt(np.sum(a.reshape(-1, ref[f"level_{k}"].size) ** 2, axis=0))
        lr = ref[f"level_{k}"]
        e_lev = float(np.max(np.abs(lv - lr)) / max(float(np.max(lr)), 1e-300))
        e_norm = abs(float(np.linalg.norm(flat)) - nref) / scale
        out[k] = {"proj": e_proj, "sample": e_samp, "level": e_lev, "norm": e_norm}
    return out
