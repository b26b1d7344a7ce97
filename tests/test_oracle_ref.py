"""The oracle (oracle/centre_oracle.c) against the reference's own numeric
code compiled from source (oracle/_ref/libcentre_ref.so) on fresh seeded
inputs, beyond the stored fixtures: bins and extremes bit-identical,
entropies within 1e-12 relative, spanning trees identical.

Runs only where the reference checkout is present (the `ref` fixture builds
the shim through oracle/Makefile and skips otherwise)."""
import numpy as np
import pytest

from centre_gb300.synth import chain_trajectory


def _blocks(natoms, nframes, seed):
    tr = chain_trajectory(natoms, nframes, seed=seed)
    return list(tr.blocks())


@pytest.mark.parametrize("nframes,schemes", [(9_001, [30]), (4_000, [50, 7, 255])])
def test_discretize_matches_reference(orc, ref, nframes, schemes):
    for typ, blk in _blocks(7, nframes, seed=nframes):
        for opt in ((True, False) if typ == 3 else (True,)):
            ob, oe = orc.discretize(typ, blk, schemes, bins_ref=schemes[0], optimize=opt)
            rb, re = ref.discretize(typ, blk, schemes, bins_ref=schemes[0], optimize=opt)
            assert np.array_equal(ob, rb), (typ, opt)
            assert np.array_equal(oe[:, [0, 1, 3]], re[:, [0, 1, 3]]), (typ, opt)
            np.testing.assert_allclose(oe[:, 2], re[:, 2], rtol=1e-12)


@pytest.mark.parametrize("jac", [False, True])
def test_entropies_match_reference(orc, ref, jac):
    schemes, nsteps, ests = [20, 9], 3, [0, 1, 2, 3]
    bins, ext, types = [], [], []
    for typ, blk in _blocks(6, 6_007, seed=41):
        b, e = orc.discretize(typ, blk, schemes)
        bins.append(b)
        ext.append(e)
        types += [typ] * len(b)
    bins, ext, types = np.concatenate(bins), np.concatenate(ext), np.array(types, np.uint8)
    s1 = orc.entropy1d(types, bins, ext, nsteps, schemes, ests, jac)
    for d in range(len(bins)):
        r = ref.entropy1d(int(types[d]), bins[d], ext[d, 0], ext[d, 1], nsteps, schemes, ests,
                          jac)
        np.testing.assert_allclose(s1[d], r, rtol=1e-12, atol=1e-14)
    rng = np.random.default_rng(5)
    pairs = np.array(sorted({tuple(sorted(rng.choice(len(bins), 2, replace=False)))
                             for _ in range(40)}), np.uint32)
    s2 = orc.entropy2d(pairs, types, bins, ext, nsteps, schemes, ests, jac)
    for q, (i, j) in enumerate(pairs):
        r = ref.entropy2d(int(types[i]), int(types[j]), bins[i], bins[j], ext[i], ext[j], nsteps,
                          schemes, ests, jac)
        np.testing.assert_allclose(s2[q], r, rtol=1e-12, atol=1e-14)


def test_mst_matches_reference(orc, ref):
    rng = np.random.default_rng(23)
    for g in range(8):
        nv = int(rng.integers(4, 60))
        E = [(i, j) for i in range(nv) for j in range(i + 1, nv) if g % 2 or rng.random() < 0.3]
        src = np.array([e[0] for e in E], np.uint32)
        dst = np.array([e[1] for e in E], np.uint32)
        w = (rng.integers(0, 5, len(E)) * 0.5) if g % 3 == 0 else rng.random(len(E))
        ts, td, _ = ref.mst(nv, src, dst, w)
        mine = orc.mst(nv, src, dst, w)
        want = {(min(a, b), max(a, b)) for a, b in zip(ts.tolist(), td.tolist())}
        got = {(int(src[k]), int(dst[k])) for k in mine.tolist()}
        assert got == want, g


def test_vmkde_matches_reference(orc, ref):
    tr = chain_trajectory(6, 5_000, seed=77)
    for kappa, nconf in ((1.0, 5), (8.0, 3)):
        for d in range(len(tr.torsions)):
            ob, om, of = orc.vmkde(tr.torsions[d], nconf, kappa, 5, 1e-4, 1000)
            rb, rm, rf = ref.vmkde(tr.torsions[d], nconf, kappa, 5, 1e-4, 1000)
            assert of == rf
            assert np.array_equal(om, rm)
            assert np.array_equal(ob, rb)


def test_bessel_matches_reference(orc, ref):
    for n in (0, 1, 2, 3):
        for x in (0.1, 1.0, 3.75, 8.0, 50.0, 100.0):
            assert orc.bessel_i(n, x) == ref.bessel_i(n, x), (n, x)
