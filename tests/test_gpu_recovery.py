"""Neighbour-list overflow and NaN during a run (src/neighborlist.cpp:247-297,
src/md_simulator.cpp:646-652).

The reference's list is a vector of vectors and cannot overflow; the device list
has a fixed number of slots per atom.  A build that wants more halts the chunk of
steps (every later kernel of the chunk returns at once), the host sees it in the
status words it reads after every chunk, grows the list, builds it again from
the same positions and completes the step.  The run must then equal, bit for
bit, a run whose list never overflowed.  Here an FCC lattice at rho 0.65 (54
neighbours per atom within r_c + skin at set-up, under the 64 slots asked for)
melts at T 1.44 and its largest neighbour count climbs past 64 during the run.

A NaN acceleration ends the run with CAVGPU_E_NAN at the step that met it, as the
reference ends there; a context that met one does not step again.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


def melting_lattice():
    pos, vel, typ, p = W.lj_fluid((10, 10, 10), rho=0.65, temperature=1.44, seed=2024)
    return pos, vel, typ, p


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED], ids=["fp64", "mixed"])
def test_overflow_mid_run_equals_large_list_run(precision):
    pos, vel, typ, p = melting_lattice()
    runs = {}
    for cap in (64, 512):
        s = G.System(pos, vel, typ, p, precision=precision, nbr_capacity=cap)
        s.setup()
        assert s.stats()["capacity"] == cap  # the set-up build fits (54 neighbours)
        th = s.run(600, 10)
        st = s.stats()
        runs[cap] = (s.state(), th, st)
        s.close()
    (p64, v64, a64), th64, st64 = runs[64]
    (pbig, vbig, abig), thbig, stbig = runs[512]
    assert st64["max_neighbours"] > 64, st64  # the run did overflow the small list
    assert st64["capacity"] > 64
    assert st64["steps"] == stbig["steps"] == 600
    assert st64["rebuilds"] == stbig["rebuilds"]
    np.testing.assert_array_equal(p64, pbig)
    np.testing.assert_array_equal(v64, vbig)
    np.testing.assert_array_equal(a64, abig)
    np.testing.assert_array_equal(th64, thbig)


@pytest.mark.parametrize("every", [3, 7])
def test_overflow_records_stay_on_their_steps(every):
    """After a completed overflow step the run resumes at a step that need not end a
    record period; the records must still fall on steps every, 2 every, ... (a
    chunk that resumes mid-period runs up to the next record first)."""
    pos, vel, typ, p = melting_lattice()
    runs = {}
    for cap in (64, 512):
        s = G.System(pos, vel, typ, p, precision=G.FP64, nbr_capacity=cap)
        s.setup()
        th = s.run(600, every)
        runs[cap] = (th, s.stats(), s.state())
        s.close()
    assert runs[64][1]["capacity"] > 64  # the small list overflowed during the run
    np.testing.assert_array_equal(runs[64][0], runs[512][0])
    for a, b in zip(runs[64][2], runs[512][2]):
        np.testing.assert_array_equal(a, b)


def test_nan_ends_the_run_at_its_step():
    pos, vel, typ, p = W.lj_fluid((5, 5, 5), seed=3)
    pos = pos.copy()
    pos[7] = pos[3]  # two atoms at one point: their pair force is NaN from the set-up on
    s = G.System(pos, vel, typ, p, precision=G.FP64)
    s.setup()
    _, _, a = s.state()
    assert np.isnan(a[3]).any() and np.isnan(a[7]).any()
    with pytest.raises(G.CavError) as e:
        s.step(200)
    assert e.value.status == G.E_NAN
    assert s.stats()["steps"] == 0  # the first step's drift met the NaN acceleration
    with pytest.raises(G.CavError) as e:
        s.step(5)
    assert e.value.status == G.E_NAN
    s.close()
