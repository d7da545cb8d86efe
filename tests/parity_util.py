"""Helpers shared by the parity tests: build the same case in the oracle and
on the GPU, and compare their state array by array."""
from __future__ import annotations

import numpy as np

FIELDS = ("u", "v", "w", "p", "ut", "vt", "wt")


def bits(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    return a.view(np.uint64) if a.dtype == np.float64 else a


def assert_bitwise(name: str, ref: np.ndarray, got: np.ndarray):
    ref = np.asarray(ref)
    got = np.asarray(got).reshape(ref.shape, order="F") if got.size == ref.size else np.asarray(got)
    assert ref.shape == got.shape, f"{name}: shape {ref.shape} vs {got.shape}"
    rb, gb = bits(np.asfortranarray(ref).ravel(order="F")), bits(np.asfortranarray(got).ravel(order="F"))
    bad = np.nonzero(rb != gb)[0]
    if bad.size:
        q = bad[0]
        idx = np.unravel_index(q, ref.shape, order="F")
        raise AssertionError(
            f"{name}: {bad.size} of {rb.size} entries differ; first at {tuple(int(i) + 1 for i in idx)} "
            f"(1-based): oracle {ref.ravel(order='F')[q]!r} gpu {got.ravel(order='F')[q]!r}")


def rel_l2(ref: np.ndarray, got: np.ndarray) -> float:
    den = float(np.linalg.norm(ref.ravel()))
    return float(np.linalg.norm((got - ref).ravel())) / (den if den > 0 else 1.0)


def compare_fields(o, s, tag: str, exact: bool = True, tol: float = 0.0):
    for gi, g in enumerate(s.handles, 1):
        f = s.fields(g)
        for nm in FIELDS:
            if exact:
                assert_bitwise(f"{tag} block {gi} {nm}", o.arr(gi, nm), f[nm])
            else:
                e = rel_l2(o.arr(gi, nm), f[nm])
                assert e <= tol, f"{tag} block {gi} {nm}: rel L2 {e:.3e} > {tol:.1e}"


def compare_search(o, s, tag: str):
    for gi, (g, spec) in enumerate(zip(s.handles, s.case.blocks), 1):
        t = s.tags(g)
        for nm in ("cell", "cell2", "nodeIdTag", "cell_n", "cell_pr"):
            assert_bitwise(f"{tag} block {gi} {nm}", o.arr(gi, nm), t[nm])
        if not spec.has_body:
            continue
        c = s.counts(g)
        for k in ("ibCellCount", "solidCellCount", "fluidCellCount", "redCellCount", "blackCellCount",
                  "TSCellCount"):
            assert c[k] == o.geti(gi, k), f"{tag} block {gi} {k}: {o.geti(gi, k)} vs {c[k]}"
        nib = c["ibCellCount"]
        assert_bitwise(f"{tag} block {gi} interceptedIndexPtr", o.arr(gi, "interceptedIndexPtr"),
                       s.read_list(g, "interceptedIndexPtr", nib))
        for nm in ("nelp", "nelu1", "nelu2", "nelv1", "nelv2", "nelw1", "nelw2"):
            assert_bitwise(f"{tag} block {gi} {nm}", o.arr(gi, nm), s.read(g, nm, nib, np.int64))
        for nm in ("pNormDis", "u1NormDis", "u2NormDis", "v1NormDis", "v2NormDis", "w1NormDis", "w2NormDis"):
            assert_bitwise(f"{tag} block {gi} {nm}", o.arr(gi, nm), s.read(g, nm, nib))


def compare_iters(o, s, tag: str):
    for gi, g in enumerate(s.handles, 1):
        n, d2, ds = s.sor_stats(g)
        assert n == o.geti(gi, "nIterPcor"), f"{tag} block {gi}: SOR iterations {o.geti(gi, 'nIterPcor')} vs {n}"
        assert_bitwise(f"{tag} block {gi} derr2", np.array([o.getf(gi, "derr2")]), np.array([d2]))
        assert_bitwise(f"{tag} block {gi} derrStdSt", np.array([o.getf(gi, "derrStdSt")]), np.array([ds]))
