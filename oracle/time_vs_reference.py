"""Speed of the oracle (the C restatement timed as the CPU baseline) against
the reference's own compiled numeric code, on the same pairs, one thread each.

TEST INFRASTRUCTURE ONLY.  Needs the reference checkout (oracle/_ref built
by `make -C oracle ref`), so it runs where the reference sources are, not on
the GPU machine.  It states how far the timed CPU baseline (the restatement)
is from the reference's own binData2D + entropy2D (src/Estimators.cpp:130-205,
391-651), which forms each joint index with pow() per frame, built twice: with
the flags the parity tests use (-O2) and with the reference's release flags
(-Ofast, configure.ac:87).

    python oracle/time_vs_reference.py [npairs] [nframes]
"""
from __future__ import annotations

import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from centre_gb300.synth import chain_trajectory  # noqa: E402


def main(npairs: int = 60, nframes: int = 100_000, nbins: int = 50, nsteps: int = 10):
    oracle.build(with_ref=True)
    if not oracle.ref_available():
        sys.exit("reference shim not built (no reference checkout)")
    subprocess.run(["make", "-s", "-C", HERE, "ref-ofast"], check=True)
    orc, ref = oracle.Oracle(), oracle.Reference()
    fast = oracle.Reference(os.path.join(HERE, "_ref", "libcentre_ref_ofast.so"))
    tr = chain_trajectory(20, nframes, seed=5, coupling="block8")
    bins, ext, types = [], [], []
    for typ, blk in tr.blocks():
        b, e = orc.discretize(typ, blk, [nbins])
        bins.append(b)
        ext.append(e)
        types += [typ] * len(b)
    bins, ext, types = np.concatenate(bins), np.concatenate(ext), np.array(types, np.uint8)
    rng = np.random.default_rng(1)
    pairs = np.array([sorted(rng.choice(len(types), 2, replace=False)) for _ in range(npairs)],
                     np.uint32)
    res = {}
    for rep in range(2):   # second repetition is the one reported (warm caches)
        t0 = time.perf_counter()
        so = orc.entropy2d(pairs, types, bins, ext, nsteps, [nbins], [0], True, nthreads=1)
        t_orc = time.perf_counter() - t0
        t0 = time.perf_counter()
        sr = np.stack([ref.entropy2d(int(types[i]), int(types[j]), bins[i], bins[j], ext[i],
                                     ext[j], nsteps, [nbins], [0], True) for i, j in pairs])
        t_ref = time.perf_counter() - t0
        t0 = time.perf_counter()
        sf = np.stack([fast.entropy2d(int(types[i]), int(types[j]), bins[i], bins[j], ext[i],
                                      ext[j], nsteps, [nbins], [0], True) for i, j in pairs])
        t_fast = time.perf_counter() - t0
        res = {"orc": t_orc, "ref": t_ref, "fast": t_fast}
    np.testing.assert_allclose(so, sr, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(so, sf, rtol=1e-9, atol=1e-12)
    ms = {k: 1e3 * v / npairs for k, v in res.items()}
    print(f"{npairs} pairs x {nframes} frames, {nbins} bins, {nsteps} steps, one thread: "
          f"oracle {ms['orc']:.3f} ms/pair; reference -O2 {ms['ref']:.3f} ms/pair "
          f"({ms['ref'] / ms['orc']:.2f}x the oracle); reference -Ofast {ms['fast']:.3f} "
          f"ms/pair ({ms['fast'] / ms['orc']:.2f}x the oracle)")


if __name__ == "__main__":
    a = [int(x) for x in sys.argv[1:3]]
    main(*a)
