"""CPU: workload generators and host-side scheduling logic."""
import numpy as np

from pycd_gb300 import workloads as wl
from pycd_gb300.autotune import candidates
from pycd_gb300.serving import poisson_jobs


def test_supercells_hold_the_cutoff_and_target_sizes():
    for lattice, per in (("corundum", 12), ("monoclinic", 4)):
        for target in (300, 1000, 2000, 7000, 20000, 50000):
            s = wl.supercell_for(lattice, target)
            assert s[0] == s[1] and s[0] >= 3
            assert s[2] >= (1 if lattice == "corundum" else 3)
            n = per * s[0] * s[1] * s[2]
            assert 0.5 * target < n < 2.0 * target


def test_uneven_batch_is_seeded_and_in_range():
    a = wl.uneven_systems()
    b = wl.uneven_systems()
    assert [x["cells"] for x in a[0]] == [x["cells"] for x in b[0]]
    specs, traj_sys, steps = a
    assert len(specs) == 64 and len(traj_sys) == 2048
    assert all(1 <= s["carriers"] <= 16 and 0 <= s["dopants"] <= 16 for s in specs)
    assert steps.min() >= 10_000 and steps.max() <= 1_000_000
    assert {s["lattice"] for s in specs} == {"corundum", "monoclinic"}


def test_poisson_arrivals_statistics():
    jobs = poisson_jobs(4000, rate=200.0, seed=1)
    gaps = np.diff([j["arrival"] for j in jobs])
    assert abs(gaps.mean() - 1 / 200.0) < 0.1 / 200.0
    assert all(1 <= j["carriers"] <= 32 for j in jobs)
    assert all(10_000 <= j["steps"] <= 1_000_000 for j in jobs)
    assert len({j["id"] for j in jobs}) == 4000


def test_autotune_candidates_respect_kernel_limits():
    for npr, nc in ((4, 1), (16, 4), (64, 16), (128, 32), (96, 32)):
        cands = candidates(npr, nc)
        for c in cands:
            lanes = c["lanes_per_traj"]
            assert lanes >= nc and -(-npr // lanes) <= 8
            # the register-capped instances exist for <= 2 processes per lane
            assert c["min_blocks_per_sm"] == 1 or -(-npr // lanes) <= 2
            # block-per-trajectory instances: 2 or 4 warps, <= 4 processes per lane
            if lanes > 32:
                assert lanes in (64, 128) and c["warps_per_block"] == lanes // 32
                assert -(-npr // lanes) <= 4 and npr > 32
        assert any(c["lanes_per_traj"] > 32 for c in cands) == (npr > 32)


def test_monoclinic_hop_shells_have_three_neighbours():
    s = wl.monoclinic((3, 3, 3), 0.9164, neighbor_list=True)
    assert int(s.num_neighbors[0]) == 3
    run = wl.run_for(s, 2)
    assert run.n_slots == 3 and (run.site_nbr >= 0).all()
