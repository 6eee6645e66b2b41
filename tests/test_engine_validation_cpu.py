"""Input validation of the engine and the surrogate on the host (no GPU).

Every check below fails before any device call, with a message the caller can read
(cgppd_get_last_error -> CgppdError): the library reports bad input instead of faulting.
"""
import numpy as np
import pytest

import cgppd_gb300
from cgppd_gb300 import CgppdError
from cgppd_gb300 import engine as eng


@pytest.fixture(scope="module", autouse=True)
def built():
    cgppd_gb300.build()


def table(n=20):
    rng = np.random.default_rng(0)
    t = rng.uniform(-3, 1, size=(n, n)).astype(np.float32)
    return (t + t.T) / 2


def chain(n):
    x = np.zeros((n, 3), np.float32)
    x[:, 0] = 3.8 * np.arange(n)
    return x


def engine_with(box=100.0, types=None, nrep=2):
    e = eng.Engine(table())
    s = e.add_simulation(np.full(nrep, 300.0), np.full(nrep, 1.0), np.full(nrep, 0.2), box)
    n = 5
    e.add_molecule(s, chain(n), types if types is not None else np.arange(n), np.zeros(n), np.full(n, 5.0))
    return e


def test_contact_table_size_is_checked():
    with pytest.raises(CgppdError, match="1..32 types"):
        eng.Engine(np.zeros((33, 33), np.float32))


def test_replica_ladders_are_required():
    e = eng.Engine(table())
    with pytest.raises(CgppdError, match="ladders"):
        e.add_simulation([], [], [], 100.0)


def test_segment_residues_are_checked():
    e = eng.Engine(table())
    s = e.add_simulation([300.0], [1.0], [0.2], 100.0)
    with pytest.raises(CgppdError, match="segment residue out of range"):
        e.add_molecule(s, chain(5), np.arange(5), np.zeros(5), np.full(5, 5.0), segments=[[3, 4, 5]])


def test_residue_types_are_checked_at_finalize():
    e = engine_with(types=np.array([0, 1, 2, 3, 20]))
    with pytest.raises(CgppdError, match="residue type outside the contact table"):
        e.finalize(1, 256)


def test_box_must_be_positive():
    e = engine_with(box=0.0)
    with pytest.raises(CgppdError, match="box edge must be positive"):
        e.finalize(1, 256)


def test_run_needs_a_finalized_engine():
    e = engine_with()
    with pytest.raises(CgppdError, match="not finalized"):
        e.run(1, 10)


def test_surrogate_batch_must_be_a_multiple_of_128():
    from cgppd_gb300 import surrogate as sg
    with pytest.raises(CgppdError, match="multiple of 128"):
        sg.Surrogate(batch=100)


def crowded_engine(order, flexible_crowder=False):
    e = eng.Engine(table())
    s = e.add_simulation([300.0, 310.0], [1.0, 1.0], [0.2, 0.2], 100.0, repulsive_crowding=True)
    for k, crowder in enumerate(order):
        x = chain(6) + np.float32(20.0 * k)
        e.add_molecule(s, x, np.arange(6), np.zeros(6), np.full(6, 5.0), crowder=crowder,
                       all_flexible=flexible_crowder and crowder)
    return e


def test_repulsive_crowding_needs_trailing_crowders():
    e = crowded_engine([False, True, False])
    with pytest.raises(CgppdError, match="crowders after every other molecule"):
        e.finalize(1, 256)


def test_repulsive_crowding_needs_rigid_crowders():
    e = crowded_engine([False, True], flexible_crowder=True)
    with pytest.raises(CgppdError, match="rigid crowders"):
        e.finalize(1, 256)
