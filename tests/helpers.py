"""Shared comparison helpers for the parity tests."""
import numpy as np

TWO_PI = 2 * np.pi


def cplx(pairs):
    a = np.asarray(pairs, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def branch_distance(im_a, im_b, n):
    """Distance of n*Im(ln det/n) values modulo 2 pi (the reference's Im part is
    sum Arg U_ii + pi[odd], which equals arg det only modulo 2 pi)."""
    d = (np.asarray(im_a) - np.asarray(im_b)) * n
    return np.abs((d + np.pi) % TWO_PI - np.pi)


def match_root_sets(got, want, tol):
    """Every wanted root has a distinct found root within tol*|k| (set semantics
    of the reference's assert_cvector_subset, src/test/assertion.c:136)."""
    got = list(np.asarray(got))
    bad = []
    for w in np.asarray(want):
        if not got:
            bad.append(w)
            continue
        dist = np.abs(np.asarray(got) - w)
        j = int(np.argmin(dist))
        if dist[j] <= tol * max(abs(w), 1.0):
            got.pop(j)
        else:
            bad.append(w)
    return bad
