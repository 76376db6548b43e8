"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark workloads (no dataset files exist on either machine).

* ``uniform``      -- i.i.d. U[0,1) float32 corpus and queries (65,536 x 128,
                      1,024 queries, k=16 workload; also the reference demos'
                      ``single(rand(d, N))`` inputs, demo/knnTest.m:23-24).
* ``int_descriptor`` -- integer-valued float32: clip(round(|N(0,40)|), 0, 255)
                      with exactly round(0.08*d) coordinates of every row set
                      to 0 at uniformly drawn positions (1,000,000 x 128,
                      10,000 queries, k=100 workload).
* ``gauss_mixture`` -- 1,024-centre isotropic Gaussian mixture, centres
                      N(0,1), sigma 0.15, rows L2-normalised.
* ``anisotropic``   -- N(0, diag(s)), s_j = 1/(1+j)^0.5.
"""
from __future__ import annotations

import numpy as np


def uniform(n, d, seed=0, nq=0):
    rng = np.random.default_rng(seed)
    corpus = rng.random((n, d), dtype=np.float32)
    queries = rng.random((nq, d), dtype=np.float32)
    return corpus, queries


def _int_rows(rng, n, d, chunk=131072):
    out = np.empty((n, d), np.float32)
    nz = int(round(0.08 * d))
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        x = np.clip(np.rint(np.abs(rng.normal(0.0, 40.0, (m, d)))), 0, 255).astype(np.float32)
        if nz:
            pos = np.argpartition(rng.random((m, d)), nz - 1, axis=1)[:, :nz]
            np.put_along_axis(x, pos, 0.0, axis=1)
        out[s:s + m] = x
    return out


def int_descriptor(n, d, seed=1, nq=0):
    rng = np.random.default_rng(seed)
    corpus = _int_rows(rng, n, d)
    queries = _int_rows(rng, nq, d)
    return corpus, queries


def gauss_mixture(n, d, seed=2, nq=0, centres=1024, sigma=0.15):
    rng = np.random.default_rng(seed)
    c = rng.normal(0.0, 1.0, (centres, d)).astype(np.float32)

    def draw(m):
        lab = rng.integers(0, centres, m)
        x = c[lab] + rng.normal(0.0, sigma, (m, d)).astype(np.float32)
        x /= np.linalg.norm(x, axis=1, keepdims=True)
        return x.astype(np.float32)

    return draw(n), draw(nq)


def anisotropic(n, d, seed=3, nq=0):
    rng = np.random.default_rng(seed)
    s = (1.0 / np.sqrt(1.0 + np.arange(d))).astype(np.float32)
    corpus = (rng.standard_normal((n, d), dtype=np.float32) * np.sqrt(s)).astype(np.float32)
    queries = (rng.standard_normal((nq, d), dtype=np.float32) * np.sqrt(s)).astype(np.float32)
    return corpus, queries
