"""Synthetic lattices of the benchmark configurations.

* corundum: the 12-site Fe sublattice of hematite (hexagonal a = 5.038 A,
  c = 13.772 A, R-centred 12c sites at z = 0.3553), hop shells 2.90 / 2.97 A
  (+-0.01), lambda 0.9 eV, V_ab 0.2 eV, vn 1.85e13 /s, eps 12,
  alpha 0.25, r_cut 6.4 A, k_cut 1.6 / A, lattice charge 0, electrons -1.
  3x3x3 cells = 324 sites (plain form), 10x10x3 = 3,600 sites (batched).
* monoclinic: a = 5.195, b = 11.701, c = 5.092 A, gamma = 90.38 deg, 4 sites
  per cell, alpha 0.2; supercells (16,16,8/16/32) give 8,192-32,768 sites
  (split-precision Ewald build).

Each builder returns this package's Material / Neighbors / System objects;
``batched_tables`` turns one of them into device KMC tables with carriers
and fixed dopant charges.
"""
import tempfile
from pathlib import Path

import numpy as np

from . import constants as K
from .core import Run, System
from .io import write_poscar
from .lattice import Material, Neighbors, ReturnValues

CORUNDUM_LATTICE = [[5.038, 0.0, 0.0], [-2.519, 4.363036, 0.0], [0.0, 0.0, 13.772]]
MONOCLINIC_GAMMA = 90.38


def corundum_frac(z=0.3553):
    base = [(0, 0, z), (0, 0, -z), (0, 0, 0.5 + z), (0, 0, 0.5 - z)]
    cent = [(0, 0, 0), (2 / 3, 1 / 3, 1 / 3), (1 / 3, 2 / 3, 2 / 3)]
    return np.array([[(b[i] + c[i]) % 1.0 for i in range(3)]
                     for c in cent for b in base])


def corundum_params():
    return dict(
        name="corundum", species_types=["electron"],
        species_charge_list={"full": [-1]},
        species_to_element_type_map={"electron": ["Fe"]},
        charge_types={"full": {"Fe": 0.0}},
        neighbor_cutoff_dist={"Fe:Fe": [[2.90, 2.97]]},
        neighbor_cutoff_dist_tol={"Fe:Fe": [[0.01, 0.01]]},
        vn=1.85e13, lambda_values={"Fe:Fe": [[0.9, 0.9]]},
        v_ab={"Fe:Fe": [[0.2, 0.2]]}, class_list={"Fe": [1] * 12},
        element_type_delimiter=":", dielectric_constant=12.0,
        alpha=0.25, r_cut=6.4, k_cut=1.6)


def monoclinic_lattice():
    a, b, c = 5.195, 11.701, 5.092
    g = np.deg2rad(MONOCLINIC_GAMMA)
    return [[a, 0.0, 0.0], [b * np.cos(g), b * np.sin(g), 0.0], [0.0, 0.0, c]]


MONOCLINIC_FRAC = [[0.0, 0.125, 0.5], [0.0, 0.875, 0.5], [0.5, 0.625, 0.5],
                   [0.5, 0.375, 0.5]]


def monoclinic_params(k_cut):
    # hop shells: the first three distinct V-V distances of this cell
    # (one neighbour each at 2.9253, 3.8991 and 3.9249 A), with the corundum
    # lambda and V_ab
    return dict(
        name="monoclinic", species_types=["electron"],
        species_charge_list={"full": [-1]},
        species_to_element_type_map={"electron": ["V"]},
        charge_types={"full": {"V": 0.0}},
        neighbor_cutoff_dist={"V:V": [[2.9253, 3.8991, 3.9249]]},
        neighbor_cutoff_dist_tol={"V:V": [[0.005, 0.005, 0.005]]},
        vn=1.85e13, lambda_values={"V:V": [[0.9, 0.9, 0.9]]},
        v_ab={"V:V": [[0.2, 0.2, 0.2]]}, class_list={"V": [1] * 4},
        element_type_delimiter=":", dielectric_constant=12.0,
        alpha=0.2, r_cut=6.4, k_cut=k_cut)


def supercell_for(lattice, target_sites):
    """(s, s, t) supercell nearest to `target_sites` whose inscribed sphere
    holds the 6.4 A real-space cutoff (s_a = s_b keeps the Ewald cell equal to
    the supercell)."""
    per, s_min, t_min = (12, 3, 1) if lattice == "corundum" else (4, 3, 3)
    best = None
    for s in range(s_min, 200):
        if per * s * s * t_min > 4 * target_sites:
            break
        t = max(t_min, int(round(target_sites / (per * s * s))))
        n = per * s * s * t
        cand = (abs(np.log(n / target_sites)), (s, s, t))
        if best is None or cand < best:
            best = cand
    return best[1]


def system_for(lattice, cells):
    if lattice == "corundum":
        return corundum(cells)
    return monoclinic(cells, 0.9164, neighbor_list=True)


def uneven_systems(seed=2025, n_systems=64, n_traj=2048, min_sites=300,
                   max_sites=20000):
    """The uneven batch: seeded lattices, supercells with log-uniform site
    counts, carriers U{1..16}, dopants U{0..16}, and trajectories spread over
    the systems with step budgets U[1e4, 1e6]."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_systems):
        lattice = "corundum" if rng.random() < 0.5 else "monoclinic"
        target = float(np.exp(rng.uniform(np.log(min_sites), np.log(max_sites))))
        specs.append({"lattice": lattice, "cells": supercell_for(lattice, target),
                      "carriers": int(rng.integers(1, 17)),
                      "dopants": int(rng.integers(0, 17)), "seed": int(seed + i)})
    traj_sys = np.sort(rng.integers(0, n_systems, n_traj))
    steps = rng.integers(10_000, 1_000_001, n_traj)
    return specs, traj_sys, steps


def sites_for(n_sites, n_carriers, n_dopants, seed):
    """Distinct carrier and dopant sites from `seed`."""
    s = np.random.default_rng(seed).choice(n_sites, size=n_carriers + n_dopants,
                                           replace=False)
    return s[:n_carriers].tolist(), s[n_carriers:].tolist()


def _material(params, lattice, types_, counts, frac):
    d = Path(tempfile.mkdtemp(prefix="pycd_lattice_"))
    write_poscar(d / "POSCAR", params["name"], lattice, types_, counts, frac)
    p = dict(params)
    p["input_coord_file_location"] = d / "POSCAR"
    return Material(ReturnValues(**p))


def corundum(cells=(3, 3, 3), neighbor_list=True, shells=None):
    """The corundum Fe sublattice; `shells` replaces the two hop shells
    (2.90, 2.97 A) by the given Fe-Fe distances (2.90, 2.971, 3.364, 3.705,
    3.986 A hold 1, 3, 3, 6, 1 neighbours), each with lambda 0.9 eV and
    V_ab 0.2 eV."""
    params = corundum_params()
    if shells is not None:
        n = len(shells)
        params.update(neighbor_cutoff_dist={"Fe:Fe": [list(shells)]},
                      neighbor_cutoff_dist_tol={"Fe:Fe": [[0.01] * n]},
                      lambda_values={"Fe:Fe": [[0.9] * n]},
                      v_ab={"Fe:Fe": [[0.2] * n]})
    mat = _material(params, CORUNDUM_LATTICE, ["Fe"], [12], corundum_frac())
    nb = Neighbors(mat, np.asarray(cells), np.array([1, 1, 1]))
    hop = nb.generate_neighbor_list(None, (3, 3, 3), save=False) \
        if neighbor_list else None
    system = System(mat, nb, hop, None, params["alpha"], params["r_cut"],
                    params["k_cut"])
    return system


def monoclinic(cells, k_cut, neighbor_list=False):
    params = monoclinic_params(k_cut)
    mat = _material(params, monoclinic_lattice(), ["V"], [4], MONOCLINIC_FRAC)
    nb = Neighbors(mat, np.asarray(cells), np.array([1, 1, 1]))
    hop = nb.generate_neighbor_list(None, (3, 3, 3), save=False) \
        if neighbor_list else None
    return System(mat, nb, hop, None, params["alpha"], params["r_cut"],
                  params["k_cut"])


def run_for(system, n_carriers, t_final=1e-6, time_interval=1e-9, temp=300,
            n_traj=1, precomputed_array=None):
    """A Run of `n_carriers` electrons (explicit occupancy is set per
    trajectory by the caller, or drawn by the Run from its MT19937 stream)."""
    return Run(system, precomputed_array, temp, "full", "full", n_traj, t_final,
               time_interval,
               np.array([n_carriers]), {"electron": []},
               {"class_index": {}, "doping": {}},
               {"electric": {"active": 0, "dir": [1, 0, 0], "ld": 0, "mag": 0.0}},
               {"num_dopants": [0]})


def batched_tables(system, A_device, n_carriers, dopant_sites, dopant_charge=1.0,
                   t_final=1e-6, time_interval=1e-9):
    """Device KMC tables for `system` with fixed dopant charges (overwriting
    the lattice charge at `dopant_sites`, as charge_config does)."""
    from .kmc import KmcTables
    run = run_for(system, n_carriers, t_final, time_interval)
    q = run.base_charge_config()[:, 0].copy()
    q[list(dopant_sites)] = dopant_charge
    n_path = int(run.t_final / run.time_interval) + 1
    return KmcTables(A_device, run.site_nbr, run.site_hop, run.site_lam,
                     run.site_vab, run.system_relative_energies, q,
                     run.carrier_charge, n_carriers, run.material.vn, run.temp,
                     run.time_interval, n_path), run


def batched_uniform_sites(seed=3600, n_sites=3600, n_carriers=4, n_dopants=4):
    """Distinct seeded sites: the first n_carriers for electrons, the rest for
    +1 dopants."""
    s = np.random.default_rng(seed).choice(n_sites, size=n_carriers + n_dopants,
                                           replace=False)
    return s[:n_carriers].tolist(), s[n_carriers:].tolist()
