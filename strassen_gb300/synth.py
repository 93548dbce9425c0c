"""Seeded synthetic inputs for the block-sparse GEMM and RI-K workloads.

Every value comes from integer hashing (splitmix64) followed by IEEE-exact
double arithmetic, so numpy on any host and the C generator in
``csrc/synth.c`` produce bit-identical arrays.  "Gaussian" entries are an
Irwin-Hall sum of four uniforms rescaled to unit variance (bounded tails at
+-3.46); envelopes that need ``exp`` are evaluated on small per-block tables
that both sides share.

The configurations follow the workloads the reference is benchmarked on:

* ``decay_matrix`` -- block (I, J) of a matrix with envelope
  ``exp(-|I-J|/L)`` (optionally a dense core), as used for the screened GEMM
  and the hybrid Strassen recursion;
* ``rik_system`` -- atoms in a box, per-atom basis / auxiliary functions,
  compressed significant-pair 3-centre integrals with ``v2m`` keys
  (``key = mu + nu*N_bf``, mu <= nu), the inverse square root of an SPD
  Coulomb metric, and localized orthonormal occupied coefficients.
"""
from __future__ import annotations

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_SQRT3 = float(np.sqrt(np.float64(3.0)))


def splitmix64(x):
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = x + _GOLD
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def stream_key(seed, stream):
    """Key of an independent stream (seed, stream id)."""
    return splitmix64(splitmix64(np.uint64(seed)) ^ np.uint64(stream))


def uniform(key, idx):
    """Uniform doubles in [0, 1) at integer indices idx of stream key."""
    h = splitmix64(np.asarray(idx, dtype=np.uint64) ^ np.uint64(key))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def gauss(key, idx):
    """Unit-variance Irwin-Hall(4) deviates at indices idx."""
    i4 = np.asarray(idx, dtype=np.uint64) * np.uint64(4)
    u0 = uniform(key, i4)
    u1 = uniform(key, i4 + np.uint64(1))
    u2 = uniform(key, i4 + np.uint64(2))
    u3 = uniform(key, i4 + np.uint64(3))
    return (((u0 + u1) + (u2 + u3)) - 2.0) * _SQRT3


def gauss_matrix(seed, stream, nr, nc):
    """nr x nc column-major matrix of deviates (element index r + c*nr)."""
    key = stream_key(seed, stream)
    idx = np.arange(nr * nc, dtype=np.uint64)
    return np.asfortranarray(gauss(key, idx).reshape(nc, nr).T)


def from_block_env(seed, stream, n, m, bs, env_blocks):
    """Deviates scaled by a per-block envelope table (exact products, so the
    result is bit-identical wherever the table is)."""
    I = np.arange(n) // bs
    J = np.arange(m) // bs
    return np.asfortranarray(np.asarray(env_blocks, dtype=np.float64)[I][:, J] * gauss_matrix(seed, stream, n, m))


def decay_env(nbI, nbJ, L, core_blocks=0, core_val=1.0):
    """Per-block envelope exp(-|I-J|/L) with an optional dense core."""
    env = np.exp(-np.abs(np.arange(nbI)[:, None] - np.arange(nbJ)[None, :]) / L)
    if core_blocks:
        env[:core_blocks, :core_blocks] = core_val
    return env


def decay_matrix(seed, stream, n, m, bs, L, core=0, core_val=1.0):
    """Block (I, J) scaled by exp(-|I-J|/L); a dense core of `core` rows and
    columns gets envelope core_val."""
    I = np.arange(n) // bs
    J = np.arange(m) // bs
    nbI, nbJ = I[-1] + 1 if n else 0, J[-1] + 1 if m else 0
    benv = np.exp(-np.abs(np.arange(nbI)[:, None] - np.arange(nbJ)[None, :]) / L)
    env = benv[I][:, J]
    if core:
        env[:core, :core] = core_val
    return np.asfortranarray(env * gauss_matrix(seed, stream, n, m))


def block_mask_matrix(seed, stream, n, m, bs, density):
    """Block-Bernoulli(density) pattern with unit deviates inside kept blocks."""
    nbI, nbJ = -(-n // bs), -(-m // bs)
    keep = uniform(stream_key(seed, stream + 1), np.arange(nbI * nbJ, dtype=np.uint64)).reshape(nbJ, nbI).T < density
    I = np.arange(n) // bs
    J = np.arange(m) // bs
    return np.asfortranarray(keep[I][:, J] * gauss_matrix(seed, stream, n, m))
