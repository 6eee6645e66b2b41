"""The seeded synthetic workloads are the same on every machine.

The generator uses only elementwise IEEE double arithmetic and numpy's Generator
streams (no BLAS), so a seed must give bit-identical structures on x86 and Arm hosts.
The digests below were taken on an x86 host; the test runs anywhere (no GPU).
"""
import hashlib

import numpy as np
import pytest

from cgppd_gb300 import workloads

DIGESTS = {
    "c0": "273ff57466bcf611160d4f711cdf1da4dee4e7655d33c489fcfa5fa4de7b2074",
    "c1": "66cab24931498384b1449a442aeb01d28fce95cbad3ad60fb26c3ae1e4ca5a56",
    "c2": "8ab60f3b4daaf4f98299baa4b4c2dd2173a4162f0f9c27cf1449ed3bea848a23",
    "c4": "c3b1b9132300771eb1e0f3cbae9a8121d6a3785e3471e1f1c2f4f72ba2fd3202",
}


def digest(wl):
    h = hashlib.sha256()
    for m in wl.sims[0].molecules:
        for a in (m.xyz, m.types, m.charges, m.radii):
            h.update(a.tobytes())
    h.update(wl.lj_raw.tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("cfg", sorted(DIGESTS))
def test_generation_is_bit_reproducible(cfg):
    assert digest(workloads.make(cfg)) == DIGESTS[cfg]


@pytest.mark.parametrize("cfg", ["c0", "c1", "c2", "c4"])
def test_structures_follow_the_recipe(cfg):
    wl = workloads.make(cfg)
    sim = wl.sims[0]
    for m in sim.molecules:
        bonds = np.sqrt(((m.xyz[1:].astype(np.float64) - m.xyz[:-1]) ** 2).sum(1))
        assert np.allclose(bonds, workloads.BOND, atol=1e-4)
        if m.n > 2:
            d = np.sqrt(((m.xyz[:, None, :].astype(np.float64) - m.xyz[None]) ** 2).sum(-1))
            sep = np.abs(np.arange(m.n)[:, None] - np.arange(m.n)[None])
            assert d[sep >= 3].min() >= 3.99      # self-avoiding at 4 A
            assert d[sep == 2].min() >= 3.7       # (3.7 at the c1 linker/domain joint)
    charges = np.concatenate([m.charges for m in sim.molecules if not m.crowder])
    assert 0.05 < np.mean(charges > 0) < 0.2 and 0.05 < np.mean(charges < 0) < 0.2
    assert np.all(wl.lj_raw == wl.lj_raw.T)
