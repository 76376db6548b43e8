"""Generate the known-answer fixtures in tests/golden/ (run from the repo root).

The reference ships no golden vectors for its kNN path.  These fixtures are
known answers of demo/knn.m (rank by ||y||^2 - 2 y.x with MATLAB's stable
sort, keep k, add ||x||^2) on data whose arithmetic is exact in float32, so
the answer is unique and does not depend on summation order.  They are
computed here with numpy only, independently of the C oracle and of the CUDA
engine, and every one of them holds exact ties that the lower-index rule
must break.

    python tests/golden/make_golden.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def knn_m(X, Y, k):
    """demo/knn.m with X = queries (Q x d), Y = corpus (N x d) as rows."""
    X = X.astype(np.float64)
    Y = Y.astype(np.float64)
    keys = (Y * Y).sum(1)[None, :] - 2.0 * (X @ Y.T)          # exact for these inputs
    order = np.argsort(keys, axis=1, kind="stable")[:, :k]
    D = np.take_along_axis(keys, order, axis=1) + (X * X).sum(1)[:, None]
    return D.astype(np.float32), order.astype(np.int32)


def merge_replace_max(dist, idx):
    """src/cuknnBitonic.cu:381-417 semantics, [list][q][k] -> merged list 0."""
    dist = dist.copy()
    idx = idx.copy()
    L, Q, k = dist.shape
    for s in range(Q):
        row, irow = dist[0, s], idx[0, s]
        m = int(np.argmax(row))          # first maximum
        for l in range(1, L):
            for j in range(k):
                if dist[l, s, j] < row[m]:
                    row[m] = dist[l, s, j]
                    irow[m] = idx[l, s, j]
                    m = int(np.argmax(row))
    return dist[0], idx[0]


def main():
    cases = {}
    # 1) hand-checkable: unit square corners; the centre query ties all four
    Y = np.array([[0, 0], [1, 0], [0, 1], [1, 1]], np.float32)
    X = np.array([[0, 0], [0.5, 0.5], [1, 1]], np.float32)
    cases["square"] = (Y, X, 4)
    # 2) a line with half-integer queries: every neighbour pair ties
    Y = np.arange(64, dtype=np.float32)[:, None]
    X = (np.arange(0, 64, 7) + 0.5).astype(np.float32)[:, None]
    cases["line"] = (Y, X, 9)
    # 3) small integers, many ties
    rng = np.random.default_rng(2024)
    Y = rng.integers(0, 8, (300, 6)).astype(np.float32)
    X = rng.integers(0, 8, (20, 6)).astype(np.float32)
    cases["small_int"] = (Y, X, 10)
    # 4) integer descriptors 0..255 with zeroed coordinates, d = 128, k = 100
    Y = np.clip(np.rint(np.abs(rng.normal(0, 40, (500, 128)))), 0, 255).astype(np.float32)
    X = np.clip(np.rint(np.abs(rng.normal(0, 40, (12, 128)))), 0, 255).astype(np.float32)
    for A in (Y, X):
        for r in range(A.shape[0]):
            A[r, rng.choice(128, 10, replace=False)] = 0
    cases["descriptor"] = (Y, X, 100)
    # 5) duplicated corpus rows: identical keys, lower index first
    base = rng.integers(0, 4, (10, 3)).astype(np.float32)
    Y = np.concatenate([base, base, base])
    X = base[:5].copy()
    cases["duplicates"] = (Y, X, 7)

    out = {}
    for name, (Y, X, k) in cases.items():
        D, N = knn_m(X, Y, k)
        out[f"{name}_corpus"] = Y
        out[f"{name}_queries"] = X
        out[f"{name}_k"] = np.array(k)
        out[f"{name}_dist"] = D
        out[f"{name}_idx"] = N

    # merge fixture: 3 lists of k=8 for 5 queries with ties across lists
    dl = rng.integers(0, 20, (3, 5, 8)).astype(np.float32)
    il = rng.integers(0, 1000, (3, 5, 8)).astype(np.float32)
    md, mi = merge_replace_max(dl, il)
    out.update(merge_dist_in=dl, merge_idx_in=il, merge_dist=md, merge_idx=mi)
    np.savez_compressed(os.path.join(HERE, "knn_known_answers.npz"), **out)
    print("wrote", os.path.join(HERE, "knn_known_answers.npz"), sorted(cases))


if __name__ == "__main__":
    main()
