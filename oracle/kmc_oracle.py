"""ORACLE (test infrastructure only) - CPU restatement of PyCD's KMC loop for
one trajectory with an injected stream of uniforms.  Never imported by the
product package; used by tests/, ``__graft_entry__.smoke()`` and bench.py's
``cpu_baseline`` / ``--impl reference`` legs.

Pinned: ``run`` reproduces the reference's shipped examples/Hematite and
examples/BVO trajectories from their restored MT19937 streams
(unwrapped_traj bit-identical, time_data to rounding; tests/golden) and the
reference's event stream on the 324-site corundum lattice.

It follows, with the same NumPy expressions:
  process attributes  PyCD/core.py:1946-1987 (from the hop-neighbour dict)
  process rates       PyCD/core.py:1989-2050
  selection, time     PyCD/core.py:2796-2804
  state update        PyCD/core.py:2810-2830
  path-grid rows      PyCD/core.py:2847-2861
for one carrier species on single-class hop sites or per-class tables.
"""
import numpy as np


class Tables(object):
    """Per-process lookups restated from Run.__init__ (core.py:1823-1927)
    for the single active species."""

    def __init__(self, hop_neighbor_list, key, class_of_site, n_per_cell,
                 head, total_per_cell, lam, vab, field=None):
        self.hl = hop_neighbor_list[key]
        self.class_of_site = np.asarray(class_of_site)
        self.n_per_cell, self.head, self.tpc = n_per_cell, head, total_per_cell
        self.lam, self.vab = lam, vab  # [class][hop type] in Hartree
        self.field = field

    def eei(self, site):
        return (site // self.tpc) * self.n_per_cell + (site % self.tpc - self.head)

    def processes(self, site):
        """(new site, hop vector, lambda, V_ab, field shift) per process of a
        carrier at `site`, in hop-type then neighbour order."""
        ci = self.class_of_site[site]
        e = self.eei(site)
        out = []
        for t, obj in enumerate(self.hl[ci]):
            idx = obj.neighbor_system_element_indices[e]
            vec = obj.displacement_vector_list[e]
            for j in range(len(idx)):
                sh = 0 if self.field is None else 0.5 * np.dot(self.field, vec[j])
                out.append((int(idx[j]), vec[j], self.lam[ci][t], self.vab[ci][t], sh))
        return out


def run(A, tables, occ0, q_fixed, carrier_charge, e_rel, vn, kT, uniforms,
        time_interval, n_path_steps, max_steps=None, energy0=0.0):
    """Advance one trajectory.  Returns a dict with the selected process per
    step (``proc``), the carrier site sequence (``sites``, after each step),
    ``time`` (0 then one entry per step), the path-grid ``unwrapped`` rows,
    the ``energy`` / ``delg0`` grids, ``steps`` and ``stop``
    ('done' | 'uniforms' | 'max_steps')."""
    occ = list(occ0)
    nc = len(occ)
    q = np.array(q_fixed, dtype=np.float64).reshape(-1, 1).copy()
    for s in occ:
        q[s] += carrier_charge
    unwrapped = np.zeros((n_path_steps, nc * 3))
    energy_arr = np.zeros(n_path_steps)
    delg0_arr = np.zeros(n_path_steps)
    energy = energy0
    energy_arr[0] = energy
    disp = np.zeros((1, nc * 3))
    sim_time = 0
    start = end = 1
    times = [0.0]
    procs, sites = [], []
    ui = 0
    steps = 0
    stop = "done"
    while end < n_path_steps:
        if max_steps is not None and steps >= max_steps:
            stop = "max_steps"
            break
        if ui + 2 > len(uniforms):
            stop = "uniforms"
            break
        old, new, lam, vab, sh, hop, owner = [], [], [], [], [], [], []
        for c, site in enumerate(occ):
            for (n, h, l, v, f) in tables.processes(site):
                old.append(site); new.append(n); lam.append(l); vab.append(v)
                sh.append(f); hop.append(h); owner.append(c)
        n_proc = len(old)
        k_list = np.zeros(n_proc)
        delg = np.zeros(n_proc)
        for i in range(n_proc):
            o, n = old[i], new[i]
            term01 = np.dot(q[:, 0], (A[n, :] - A[o, :]))
            term02 = carrier_charge * (A[o, o] - A[o, n])
            d0 = 2 * carrier_charge * (term01 + term02) + (e_rel[n] - e_rel[o])
            delg[i] = d0
            dgs = (((lam[i] + d0) ** 2 / (4 * lam[i])) - vab[i]) - sh[i]
            k_list[i] = vn * np.e ** (-dgs / kT)
        k_total = sum(k_list)
        k_cum = (k_list / k_total).cumsum()
        u1 = uniforms[ui]
        p = int(np.where(k_cum > u1)[0][0])
        u2 = uniforms[ui + 1]
        ui += 2
        sim_time -= np.log(u2) / k_total
        end = int(sim_time / time_interval)
        delg0_arr[start:end] = delg[p]
        c = owner[p]
        o = occ[c]
        occ[c] = new[p]
        disp[0, 3 * c:3 * c + 3] += hop[p]
        energy += delg[p]
        q[o] -= carrier_charge
        q[new[p]] += carrier_charge
        times.append(sim_time)
        procs.append(p)
        sites.append(list(occ))
        steps += 1
        if end >= start + 1:
            if end >= n_path_steps:
                end = n_path_steps
            unwrapped[start:end] = unwrapped[start - 1] + disp
            energy_arr[start:end] = energy
            disp = np.zeros((1, nc * 3))
            start = end
    return {"proc": np.asarray(procs, dtype=np.int32),
            "sites": np.asarray(sites, dtype=np.int64).reshape(-1, nc),
            "time": np.asarray(times), "unwrapped": unwrapped,
            "energy": energy_arr, "delg0": delg0_arr, "steps": steps,
            "stop": stop, "occ": occ}
