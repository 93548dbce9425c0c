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


def decay_matrix_torch(seed, stream, n, m, bs, L, core=0, core_val=1.0, device="cuda", cols_per_chunk=2048):
    """decay_matrix generated on a torch device, bit-identical to it (the same
    envelope table, the same deviates, one double multiply per element).
    Returns an (m, n) row-major tensor, i.e. the n x m column-major matrix:
    pass ``.T`` where a column-major n x m operand is expected."""
    import torch

    nbI, nbJ = -(-n // bs), -(-m // bs)
    benv = np.exp(-np.abs(np.arange(nbI)[:, None] - np.arange(nbJ)[None, :]) / L)
    key = stream_key(seed, stream)
    out = torch.empty((m, n), dtype=torch.float64, device=device)
    rb = torch.arange(n, device=device) // bs
    r = torch.arange(n, dtype=torch.int64, device=device)
    for c0 in range(0, m, cols_per_chunk):
        c1 = min(m, c0 + cols_per_chunk)
        c = torch.arange(c0, c1, dtype=torch.int64, device=device)
        idx = r[None, :] + c[:, None] * n  # [c, r] = r + c n
        env_c = torch.from_numpy(np.ascontiguousarray(benv[:, np.arange(c0, c1) // bs].T)).to(device)  # [c, I]
        env = env_c[:, rb]
        if core:
            cc = min(core, c1) - c0
            if cc > 0:
                env[:cc, :core] = core_val
        out[c0:c1] = env * gauss_torch(key, idx)
    return out


def block_mask_matrix(seed, stream, n, m, bs, density):
    """Block-Bernoulli(density) pattern with unit deviates inside kept blocks."""
    nbI, nbJ = -(-n // bs), -(-m // bs)
    keep = uniform(stream_key(seed, stream + 1), np.arange(nbI * nbJ, dtype=np.uint64)).reshape(nbJ, nbI).T < density
    I = np.arange(n) // bs
    J = np.arange(m) // bs
    return np.asfortranarray(keep[I][:, J] * gauss_matrix(seed, stream, n, m))


def _torch_splitmix64(x):
    """splitmix64 on int64 torch tensors (two's-complement wraparound gives the
    uint64 bits; logical shifts are emulated by masking)."""
    import torch

    def srl(v, k):
        return (v >> k) & ((1 << (64 - k)) - 1)

    gold = int(np.int64(np.uint64(0x9E3779B97F4A7C15).view(np.int64)))
    m1 = int(np.int64(np.uint64(0xBF58476D1CE4E5B9).view(np.int64)))
    m2 = int(np.int64(np.uint64(0x94D049BB133111EB).view(np.int64)))
    z = x + gold
    z = (z ^ srl(z, 30)) * m1
    z = (z ^ srl(z, 27)) * m2
    return z ^ srl(z, 31)


def gauss_torch(key, idx):
    """`gauss` on a torch int64 index tensor (any device); bit-identical to the
    numpy version."""
    import torch

    k = int(np.int64(np.uint64(key).view(np.int64)))
    i4 = idx * 4
    acc = []
    for j in range(4):
        h = _torch_splitmix64((i4 + j) ^ k)
        u = ((h >> 11) & ((1 << 53) - 1)).to(torch.float64) * (1.0 / 9007199254740992.0)
        acc.append(u)
    return (((acc[0] + acc[1]) + (acc[2] + acc[3])) - 2.0) * _SQRT3


class RikSystem:
    """Synthetic RI-K inputs: atoms in a cubic box, `nbf` basis and `naux`
    auxiliary functions per atom, significant (mu <= nu) pairs kept where
    exp(-r_ab^2/2) >= sig.  Integrals (mu nu|P) = exp(-(r_ab^2 + r_ap^2)/2) *
    deviate, the Coulomb metric's inverse square root from a random SPD matrix
    with a geometric spectrum of the given condition number, and localized
    occupied orbitals (Gaussian envelope around a centre atom, orthonormalized
    by QR)."""

    def __init__(self, seed=42, n_atoms=40, nbf=24, naux=84, n_occ=200, box=12.0, sig=1e-10, cond=1e4, width=2.0):
        self.seed, self.n_atoms, self.nbf, self.naux, self.box = seed, n_atoms, nbf, naux, box
        self.n_bf, self.n_aux, self.n_occ = n_atoms * nbf, n_atoms * naux, n_occ
        key = stream_key(seed, 1000)
        self.pos = uniform(key, np.arange(3 * n_atoms, dtype=np.uint64)).reshape(n_atoms, 3) * box
        d = self.pos[:, None, :] - self.pos[None, :, :]
        self.r2 = (d * d).sum(axis=2)
        self.pair_env = np.exp(-0.5 * self.r2)
        atom = np.arange(self.n_bf) // nbf
        mu, nu = np.triu_indices(self.n_bf)  # row-major upper triangle: mu <= nu
        keep = self.pair_env[atom[mu], atom[nu]] >= sig
        mu, nu = mu[keep], nu[keep]
        order = np.lexsort((mu, nu))  # column-major: by nu, then mu
        self.mu, self.nu = mu[order], nu[order]
        self.keys = (self.mu + self.nu * self.n_bf).astype(np.uint64)
        self.n_vec2 = len(self.keys)
        self.a_of_v = atom[self.mu]
        self.b_of_v = atom[self.nu]
        # (a, b, p) envelope table
        self.env3 = np.exp(-0.5 * (self.r2[:, :, None] + self.r2[:, None, :]))  # [a, b, p] = r_ab^2 + r_ap^2
        self.ints_key = stream_key(seed, 1001)

    def ints_3c(self, p_lo=0, p_hi=None):
        """columns P in [p_lo, p_hi) of the compressed (mu nu|P), n_vec2 x nP"""
        p_hi = self.n_aux if p_hi is None else p_hi
        P = np.arange(p_lo, p_hi)
        env = self.env3[self.a_of_v[:, None], self.b_of_v[:, None], (P // self.naux)[None, :]]
        idx = (np.arange(self.n_vec2, dtype=np.uint64)[:, None] + P.astype(np.uint64)[None, :] * np.uint64(self.n_vec2))
        return np.asfortranarray(env * gauss(self.ints_key, idx))

    def ints_3c_rows(self, r_lo, r_hi):
        """rows [r_lo, r_hi) of the compressed (mu nu|P) over every P"""
        v = np.arange(r_lo, r_hi)
        P = np.arange(self.n_aux)
        env = self.env3[self.a_of_v[v][:, None], self.b_of_v[v][:, None], (P // self.naux)[None, :]]
        idx = v.astype(np.uint64)[:, None] + P.astype(np.uint64)[None, :] * np.uint64(self.n_vec2)
        return np.asfortranarray(env * gauss(self.ints_key, idx))

    def ints_3c_torch(self, device, p_lo=0, p_hi=None, dtype=None):
        """the same columns generated on a torch device (bit-identical)"""
        import torch

        p_hi = self.n_aux if p_hi is None else p_hi
        env3 = torch.from_numpy(np.ascontiguousarray(self.env3)).to(device)
        a = torch.from_numpy(self.a_of_v.astype(np.int64)).to(device)
        b = torch.from_numpy(self.b_of_v.astype(np.int64)).to(device)
        out = torch.empty((p_hi - p_lo, self.n_vec2), dtype=torch.float64, device=device)  # row P = column of F-order
        v = torch.arange(self.n_vec2, dtype=torch.int64, device=device)
        for P in range(p_lo, p_hi):
            e = env3[a, b, P // self.naux]
            out[P - p_lo] = e * gauss_torch(self.ints_key, v + P * self.n_vec2)
        return out  # out.T is the column-major n_vec2 x nP matrix

    def v_m12(self, cond=1e4):
        """(P|Q)^{-1/2} of a random SPD metric with condition number `cond`"""
        n = self.n_aux
        g = gauss_matrix(self.seed, 1002, n, n)
        q, r = np.linalg.qr(g)
        q = q * np.sign(np.diag(r))[None, :]
        lam = np.geomspace(1.0, 1.0 / cond, n)
        return np.asfortranarray((q * lam ** -0.5) @ q.T)

    def c_occ(self, width=2.0):
        """localized occupied orbitals: orbital i centred on atom i % n_atoms"""
        atom = np.arange(self.n_bf) // self.nbf
        centre = np.arange(self.n_occ) % self.n_atoms
        env = np.exp(-0.5 * self.r2[atom[:, None], centre[None, :]] / width ** 2)
        c = env * gauss_matrix(self.seed, 1003, self.n_bf, self.n_occ)
        q, r = np.linalg.qr(c)
        q = q * np.sign(np.diag(r))[None, :]
        return np.asfortranarray(q)
