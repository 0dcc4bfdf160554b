"""Pattern classes of the stored ADO blocks and their same-tier (commutator) terms.

Every stored ADO keeps the entries of one sparsity pattern (fermion/prelude_spa.f90); ADOs
with equal patterns form a class, and the same-tier term -i[H, X] of every ADO of class c is
one product with the class's fixed nnz_c x nnz_c matrix L_c (from H).  Stacking the ADOs of a
class gives Y_c += X_c L_c^T, a GEMM with K = nnz_c: tensor-core shaped when nnz_c >= 16.
Counted here from the tables alone (numpy, no library plan): classes, their sizes, and the
share of the same-tier terms that falls in classes with nnz_c >= 16, for the double dot at
tier 4 and the Kanamori model at tier 2.  The GPU test checks the count against the plan the
library builds (heom_ctx_stats)."""
import numpy as np
import pytest

import heomq
from heomq import models

DSMALL = 1e-32   # the zero test of the reference (include/sizes:34)


def class_terms(m):
    """[(nnz_c, ADOs in class c, same-tier terms per ADO of c)] from the model's tables: the
    H structure is H's entries above the zero test plus the diagonal, and an entry (i, c) of
    a pattern P has one term per k with H(i, k) and (k, c) in P, and one per k with (i, k)
    in P and H(k, c)."""
    nnz, ind = m.array("nnz_spa"), m.array("ind_spa")
    ir, ic = m.array("irow_spa") - 1, m.array("icol_spa") - 1
    n = m.nrho
    H = m.array("hs").reshape(n, n, order="F")
    hnz = (np.abs(H) >= DSMALL) | np.eye(n, dtype=bool)
    classes = {}
    for u in np.nonzero(nnz)[0]:
        s = ind[u] - 1
        key = (tuple(ir[s:s + nnz[u]]), tuple(ic[s:s + nnz[u]]))
        classes[key] = classes.get(key, 0) + 1
    out = []
    for (r, c), count in classes.items():
        P = np.zeros((n, n), bool)
        P[list(r), list(c)] = True
        terms = sum(int(np.sum(hnz[i, :] & P[:, j])) + int(np.sum(P[i, :] & hnz[:, j])) for i, j in zip(r, c))
        out.append((len(r), count, terms))
    return sorted(out)


def share_in_large_classes(rows, k=16):
    tot = sum(cnt * t for _, cnt, t in rows)
    return sum(cnt * t for nz, cnt, t in rows if nz >= k) / tot, tot


@pytest.mark.parametrize("name,cfg,nclass,terms,share", [
    ("dqd_L4", models.dqd(ntier=5, nmats=3, V=0.8), 19, 1657800, 0.9089),
    ("hund_L2", models.HUND_L2, 29, 1799408, 1.0),
])
def test_same_tier_terms_by_class(name, cfg, nclass, terms, share):
    m = heomq.Model(cfg)
    rows = class_terms(m)
    assert len(rows) == nclass, name
    assert sum(nz * cnt for nz, cnt, _ in rows) == m.lunk          # every stored entry in one class
    sh, tot = share_in_large_classes(rows)
    assert tot == terms, name
    assert abs(sh - share) < 1e-4, (name, sh)
    # the classes that hold the share are few and each stacks hundreds to thousands of ADOs
    big = [(nz, cnt) for nz, cnt, _ in rows if nz >= 16]
    assert min(cnt for _, cnt in big) >= 14 and max(nz for nz, _ in big) <= 112


def class_matrix(m, nnz_c):
    """L_c of the first class with nnz_c entries: y_p = sum_q L[p, q] x_q is the same-tier term
    -i (H X - X H) restricted to the pattern (p = (i, c): -i H(i, k) on q = (k, c), +i H(k, c)
    on q = (i, k))."""
    nnz, ind = m.array("nnz_spa"), m.array("ind_spa")
    ir, ic = m.array("irow_spa") - 1, m.array("icol_spa") - 1
    n = m.nrho
    H = m.array("hs").reshape(n, n, order="F")
    u = next(u for u in np.nonzero(nnz)[0] if nnz[u] == nnz_c)
    s = ind[u] - 1
    pat = list(zip(ir[s:s + nnz_c], ic[s:s + nnz_c]))
    pos = {e: q for q, e in enumerate(pat)}
    L = np.zeros((nnz_c, nnz_c), complex)
    for p, (i, c) in enumerate(pat):
        for k in range(n):
            if (k, c) in pos:
                L[p, pos[(k, c)]] += -1j * H[i, k]
            if (i, k) in pos:
                L[p, pos[(i, k)]] += 1j * H[k, c]
    return L


def split_product(A, B, slices, bits=8):
    """A @ B by the error-free splitting of Ozaki et al. (Numer. Algorithms 59 (2012) 95): each
    row of A and each column of B is cut into `slices` pieces of `bits` significant bits
    below its largest element (exact in BF16), and the slice products with p + q <= slices + 1
    are summed.  With bits = 8 and K <= 256 every slice product sums exactly in an FP32
    accumulator, so float64 reproduces what BF16 tensor-core products with FP32 accumulation
    give."""
    def cut(M, axis):
        e = 2.0 ** np.ceil(np.log2(np.max(np.abs(M), axis=axis, keepdims=True) + 1e-300))
        out, R = [], M / e
        for k in range(1, slices + 1):
            S = np.round(R * 2.0 ** (bits * k)) / 2.0 ** (bits * k)
            out.append(S)
            R = R - S
        return out, e
    As, ea = cut(A, 1)
    Bs, eb = cut(B, 0)
    acc = np.zeros((A.shape[0], B.shape[1]))
    for p in range(slices):
        for q in range(slices - p):
            P = As[p] @ Bs[q]
            assert np.all(np.abs(P) * 2.0 ** (bits * (p + q + 2)) < 2.0 ** 24)   # exact in FP32
            acc += P
    return acc * ea * eb


def exact_product(A, B):
    from fractions import Fraction
    Af = [[Fraction(float(v)) for v in row] for row in A]
    Bf = [[Fraction(float(v)) for v in row] for row in B.T]
    return np.array([[float(sum(a * b for a, b in zip(ra, cb))) for cb in Bf] for ra in Af])


@pytest.mark.parametrize("name,cfg,nnz_c", [("dqd_L4", models.dqd(ntier=5, nmats=3, V=0.8), 36),
                                             ("hund_L2", models.HUND_L2, 112)])
def test_split_bf16_class_product_precision(name, cfg, nnz_c):
    """Can tensor-core products hold the inner solve's about 48-bit arithmetic?  The class
    product Y = X L^T in real form ([Re, Im] blocks), X random at FP64: 3 BF16 slices (what a
    BF16x3 scheme gives) leave about 2^-24 relative error; 6 slices (21 slice products) reach
    the 2^-48 of FP32x2 (measured: 2^-23.1 and 2^-46.8 on the double dot, 2^-23.5 and 2^-47.3
    on the Kanamori model).  The dense class products do sum_c n_c nnz_c^2 complex MACs, 5.6x
    (double dot) and 19x (Kanamori) the sparse terms, so the 21 slice products cost about 118x
    and 400x the sparse term count."""
    m = heomq.Model(cfg)
    L = class_matrix(m, nnz_c)
    Lr = np.block([[L.real, -L.imag], [L.imag, L.real]])              # acts on [Re x; Im x]
    X = np.random.default_rng(5).standard_normal((8, 2 * nnz_c))
    Y = exact_product(X, Lr.T)
    ref = np.linalg.norm(Y)
    e3 = np.linalg.norm(split_product(X, Lr.T, 3) - Y) / ref
    e6 = np.linalg.norm(split_product(X, Lr.T, 6) - Y) / ref
    assert 2.0 ** -30 < e3 < 2.0 ** -20, (name, e3)
    assert e6 < 2.0 ** -46, (name, e6)


@pytest.mark.gpu
def test_plan_counts_the_same_terms():
    m = heomq.Model(models.dqd(ntier=5, nmats=3, V=0.8))
    st = heomq.Context(m, adjoint=False).stats()
    rows = class_terms(m)
    assert st["classes"] == len(rows)
    assert st["same_tier_terms"] == share_in_large_classes(rows)[1]
