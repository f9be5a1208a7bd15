"""Device-side KMC: per-system tables, trajectory state and the engine that
advances them through ``pycd_kmc_advance`` (the Run.do_kmc_steps loop,
PyCD/core.py:2787-2861).

``KmcTables`` holds one lattice system in HBM: the N x N FP64 array, the
background potential phi_bg = A q_fixed, relative site energies, and the
per-(site, slot) neighbour, hop-vector, lambda, V_ab and field-shift tables
(the reference's per-process tables of core.py:1823-1927, laid out by site).
``KmcBatch`` is the structure-of-arrays state of T trajectories that may run
on different systems; the same kernel advances one trajectory (plain form) or
thousands (batched form).
"""
import ctypes as C

import numpy as np

from . import _native as nat


def _dev():
    import torch
    return torch.device("cuda", torch.cuda.current_device())


def default_lanes(max_processes, max_carriers, n_traj):
    """Lanes per trajectory the launcher picks for ``n_traj`` trajectories
    (64 or 128: one block of 2 or 4 warps per trajectory).  A batch whose
    running trajectories are fewer than its slots passes the running count
    and sets the result on its launch."""
    out = C.c_int32(0)
    nat.check(nat.lib().pycd_kmc_default_lanes(int(max_processes), int(max_carriers),
                                               int(n_traj), C.byref(out)))
    return int(out.value)


class KmcTables(object):
    """Device tables of one system (see module docstring)."""

    def __init__(self, A, nbr, hop, lam, vab, e_rel, q_fixed, carrier_charge,
                 n_carriers, vn, kT, time_interval, n_path_steps,
                 field_shift=None, phi_bg=None):
        import torch
        nat.require_device()
        dev = _dev()
        self.n_sites = int(nbr.shape[0])
        self.n_slots = int(nbr.shape[1])
        if isinstance(A, torch.Tensor):
            self.A = A.to(dev, torch.float64).contiguous()
        else:
            self.A = torch.as_tensor(np.ascontiguousarray(A, np.float64)).to(dev)
        assert tuple(self.A.shape) == (self.n_sites, self.n_sites)
        f64 = lambda x: torch.as_tensor(np.ascontiguousarray(x, np.float64)).to(dev)
        self.nbr = torch.as_tensor(np.ascontiguousarray(nbr, np.int32)).to(dev)
        self.hop = f64(hop)
        self.lam = f64(lam)
        self.vab = f64(vab)
        self.e_rel = f64(e_rel)
        self.field_shift = None if field_shift is None else f64(field_shift)
        if phi_bg is None:
            self.q_fixed = f64(q_fixed)
            self.phi_bg = torch.empty(self.n_sites, dtype=torch.float64, device=dev)
            nat.check(nat.lib().pycd_potential_gemv(
                self.A.data_ptr(), self.n_sites, self.q_fixed.data_ptr(),
                self.phi_bg.data_ptr(), None, nat.stream_handle()))
        else:
            self.phi_bg = f64(phi_bg)
        self.carrier_charge = float(carrier_charge)
        self.n_carriers = int(n_carriers)
        self.vn = float(vn)
        self.kT = float(kT)
        self.time_interval = float(time_interval)
        self.n_path_steps = int(n_path_steps)

    def with_charges(self, q_fixed, n_carriers):
        """Tables of the same lattice with other fixed charges and carrier
        count: every device tensor is shared except the new phi_bg."""
        import copy
        import torch
        t = copy.copy(self)
        q = np.ascontiguousarray(q_fixed, np.float64)
        dev = self.A.device
        t.q_fixed = torch.as_tensor(q).to(dev)
        t.phi_bg = torch.empty(self.n_sites, dtype=torch.float64, device=dev)
        nz = np.nonzero(q)[0]
        if len(nz) <= 64:  # a few charged sites: gather their rows
            d_idx = torch.as_tensor(nz.astype(np.int32)).to(dev)
            d_q = torch.as_tensor(q[nz]).to(dev)
            nat.check(nat.lib().pycd_potential_sparse(
                self.A.data_ptr(), self.n_sites, nat.ptr(d_idx), nat.ptr(d_q),
                len(nz), t.phi_bg.data_ptr(), nat.stream_handle()))
        else:
            nat.check(nat.lib().pycd_potential_gemv(
                self.A.data_ptr(), self.n_sites, t.q_fixed.data_ptr(),
                t.phi_bg.data_ptr(), None, nat.stream_handle()))
        t.n_carriers = int(n_carriers)
        return t

    def descriptor(self):
        d = nat.KmcSystem()
        d.d_A = self.A.data_ptr()
        d.d_phi_bg = self.phi_bg.data_ptr()
        d.d_e_rel = self.e_rel.data_ptr()
        d.d_nbr = self.nbr.data_ptr()
        d.d_hop = self.hop.data_ptr()
        d.d_lam = self.lam.data_ptr()
        d.d_vab = self.vab.data_ptr()
        d.d_field_shift = (self.field_shift.data_ptr()
                           if self.field_shift is not None else None)
        d.n_sites = self.n_sites
        d.n_slots = self.n_slots
        d.n_carriers = self.n_carriers
        d.carrier_charge = self.carrier_charge
        d.vn = self.vn
        d.kT = self.kT
        d.time_interval = self.time_interval
        d.n_path_steps = self.n_path_steps
        d.d_rate_coef = nat.ptr(getattr(self, "rate_coef", None))
        return d

    def share_rate_coefficients(self):
        """Compute the per-slot rate coefficients once on the device so
        every job built from these tables (``with_charges``) reuses them."""
        import torch
        if getattr(self, "rate_coef", None) is None:
            self.rate_coef = torch.empty(2 * self.n_sites * self.n_slots,
                                         dtype=torch.float64, device=self.A.device)
            d = self.descriptor()
            d.d_rate_coef = None
            nat.check(nat.lib().pycd_kmc_rate_coefficients(
                C.byref(d), self.rate_coef.data_ptr(), nat.stream_handle()))
        return self


class KmcBatch(object):
    """State of T trajectories (device SoA) plus optional outputs."""

    # exact refresh period of the carrier-potential sums (steps)
    CSUM_REFRESH = 64

    def __init__(self, occupancy, sys_index=None, max_carriers=None,
                 energy0=None, unwrapped_rows=None, step_capacity=0,
                 energy_grid_rows=None, delg0_grid_rows=None, drift=False,
                 step_limit=None, max_processes=256, cancellable=False):
        import torch
        dev = _dev()
        occ = np.asarray(occupancy, dtype=np.int32)
        if occ.ndim == 1:
            occ = occ[None, :]
        T, nc = occ.shape
        mc = max_carriers or nc
        self.n_traj, self.max_carriers = T, mc
        occ_full = np.zeros((T, mc), np.int32)
        occ_full[:, :nc] = occ
        z64 = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
        self.occ = torch.as_tensor(occ_full).to(dev)
        self.sys_index = (None if sys_index is None else
                          torch.as_tensor(np.asarray(sys_index, np.int32)).to(dev))
        self.time = z64(T)
        self.step = torch.zeros(T, dtype=torch.int64, device=dev)
        self.path_index = torch.ones(T, dtype=torch.int64, device=dev)
        self.disp = z64(T, mc * 3)
        self.last_row = z64(T, mc * 3)
        self.energy = z64(T)
        if energy0 is not None:
            self.energy.copy_(torch.as_tensor(np.asarray(energy0, np.float64)))
        self.status = torch.zeros(T, dtype=torch.int32, device=dev)
        self.u_cursor = torch.zeros(T, dtype=torch.int64, device=dev)
        self.unwrapped = (None if unwrapped_rows is None
                          else z64(T, unwrapped_rows, mc * 3))
        self.energy_grid = (None if energy_grid_rows is None
                            else z64(T, energy_grid_rows))
        if self.energy_grid is not None and energy0 is not None:
            self.energy_grid[:, 0] = self.energy
        self.delg0_grid = (None if delg0_grid_rows is None
                           else z64(T, delg0_grid_rows))
        self.step_capacity = int(step_capacity)
        self.step_time = z64(T, max(1, self.step_capacity)) if step_capacity else None
        self.step_proc = (torch.zeros(T, max(1, self.step_capacity),
                                      dtype=torch.int32, device=dev)
                          if step_capacity else None)
        self.step_offset = 0
        self.drift = z64(T, mc, 3) if drift else None
        self.step_limit = (None if step_limit is None else torch.as_tensor(
            np.broadcast_to(np.asarray(step_limit, np.int64), (T,)).copy()).to(dev))
        self.csum_stride = 2 * int(max_processes)
        self.csum = z64(T, self.csum_stride)
        self.csum_refresh = self.CSUM_REFRESH
        # cooperative stop: per-trajectory flags in pinned host memory that
        # the kernels read while they run (request_stop), and a per-launch
        # time limit (0 = none), both checked every poll_interval steps
        self.cancel = (torch.zeros(T, dtype=torch.int32, pin_memory=True)
                       if cancellable else None)
        self.time_limit_ns = 0
        self.poll_interval = 0

    def request_stop(self, t, flag=True):
        """Ask trajectory t to stop with TRAJ_CANCELLED at its next poll,
        also while a launch runs (or clear the request)."""
        if self.cancel is None:
            raise ValueError("this batch was made without cancellable=True")
        self.cancel[int(t)] = 1 if flag else 0

    def state_struct(self):
        s = nat.KmcState()
        s.n_traj = self.n_traj
        s.max_carriers = self.max_carriers
        s.d_sys_index = nat.ptr(self.sys_index)
        s.d_occ = self.occ.data_ptr()
        s.d_time = self.time.data_ptr()
        s.d_step = self.step.data_ptr()
        s.d_path_index = self.path_index.data_ptr()
        s.d_disp = self.disp.data_ptr()
        s.d_last_row = self.last_row.data_ptr()
        s.d_energy = self.energy.data_ptr()
        s.d_status = self.status.data_ptr()
        s.d_u_cursor = self.u_cursor.data_ptr()
        s.d_step_limit = nat.ptr(self.step_limit)
        s.d_csum = self.csum.data_ptr()
        s.csum_stride = self.csum_stride
        s.csum_refresh = self.csum_refresh
        s.d_cancel = nat.ptr(self.cancel)
        s.time_limit_ns = int(self.time_limit_ns)
        s.poll_interval = int(self.poll_interval)
        return s

    def outputs_struct(self):
        o = nat.KmcOutputs()
        o.d_unwrapped = nat.ptr(self.unwrapped)
        o.unwrapped_stride = (0 if self.unwrapped is None
                              else self.unwrapped.shape[1] * self.unwrapped.shape[2])
        o.d_energy_grid = nat.ptr(self.energy_grid)
        o.d_delg0_grid = nat.ptr(self.delg0_grid)
        o.d_step_time = nat.ptr(self.step_time)
        o.d_step_proc = nat.ptr(self.step_proc)
        o.step_capacity = self.step_capacity
        o.step_offset = self.step_offset
        o.d_drift = nat.ptr(self.drift)
        return o

    def snapshot(self):
        """Host copy of the resumable state (checkpoint between chunks)."""
        keys = ("occ", "time", "step", "path_index", "disp", "last_row",
                "energy", "status", "u_cursor", "csum")
        return {k: getattr(self, k).cpu().numpy().copy() for k in keys}

    def restore(self, snap):
        import torch
        for k, v in snap.items():
            getattr(self, k).copy_(torch.as_tensor(v))


class KmcEngine(object):
    """Launches ``pycd_kmc_advance`` for a set of systems and a batch."""

    def __init__(self, tables, launch=None, share=None):
        """``share``: another engine whose uploaded system table this one
        reuses (same systems, its own launch shape)."""
        import torch
        if share is not None:
            if not share._uploaded:
                share.upload()
            self.tables, self._descs = share.tables, share._descs
            self.workspace = share.workspace
            self._uploaded = True
        else:
            self.tables = (list(tables) if isinstance(tables, (list, tuple))
                           else [tables])
            self._descs = (nat.KmcSystem * len(self.tables))(
                *[t.descriptor() for t in self.tables])
            nbytes = C.c_size_t()
            nat.check(nat.lib().pycd_kmc_workspace_size(
                self._descs, len(self.tables), C.byref(nbytes)))
            self.workspace = torch.empty(nbytes.value, dtype=torch.uint8,
                                         device=_dev())
            self._uploaded = False
        self.launch = nat.KmcLaunch()
        if share is not None:
            self.launch.max_processes = share.launch.max_processes
            self.launch.max_carriers = share.launch.max_carriers
        if launch:
            for k, v in launch.items():
                setattr(self.launch, k, int(v))

    def restrict_shape(self, system_ids):
        """Size the launch for trajectories of these systems only."""
        t = [self.tables[i] for i in set(int(s) for s in system_ids)]
        self.launch.max_processes = max(x.n_carriers * x.n_slots for x in t)
        self.launch.max_carriers = max(x.n_carriers for x in t)

    def upload(self, stream=None):
        keep = (self.launch.max_processes, self.launch.max_carriers)
        nat.check(nat.lib().pycd_kmc_upload_systems(
            self._descs, len(self.tables), self.workspace.data_ptr(),
            self.workspace.numel(), nat.stream_handle(stream),
            C.byref(self.launch)))
        if keep[0] > 0:  # a restricted shape set before the upload wins
            self.launch.max_processes, self.launch.max_carriers = keep
        self._uploaded = True

    @staticmethod
    def rng_struct(uniforms=None, u_count=None, seed=0, traj_offset=0,
                   traj_ids=None):
        r = nat.KmcRng()
        r.d_traj_ids = nat.ptr(traj_ids)
        if uniforms is not None:
            r.d_uniforms = uniforms.data_ptr()
            r.u_stride = uniforms.shape[-1]
            r.u_count = uniforms.shape[-1] if u_count is None else int(u_count)
        r.seed = int(seed)
        r.traj_offset = int(traj_offset)
        return r

    def schedule(self, steps):
        """Queue form of the warp-form launches: trajectories advance in
        rounds of ``steps`` steps handed to free warps (0 = static form).
        Results do not change; the scratch is allocated on first use."""
        self.launch.sched_steps = int(steps)
        return self

    def _sched_scratch(self, batch, max_steps):
        import torch
        G = int(self.launch.lanes_per_traj or 0)
        if self.launch.sched_steps <= 0 or G > 32:
            self.launch.d_sched = None
            self.launch.sched_capacity = 0
            return
        gpw = 32 // G if G else 1  # lanes not chosen yet: one trajectory per set
        sets = -(-batch.n_traj // gpw)
        need = 4 + sets * -(-int(max_steps) // int(self.launch.sched_steps))
        buf = getattr(self, "_sched", None)
        if buf is None or buf.numel() < need:
            buf = torch.zeros(need, dtype=torch.int32, device=_dev())
            self._sched = buf
        self.launch.d_sched = buf.data_ptr()
        self.launch.sched_capacity = buf.numel()

    def advance(self, batch, max_steps, rng, stream=None):
        """Advance every running trajectory by up to ``max_steps`` steps.
        Asynchronous on ``stream``; the structs are passed by value."""
        if not self._uploaded:
            self.upload(stream)
        self._sched_scratch(batch, max_steps)
        st = batch.state_struct()
        out = batch.outputs_struct()
        nat.check(nat.lib().pycd_kmc_advance_uploaded(
            len(self.tables), C.byref(st), C.byref(out), C.byref(rng),
            int(max_steps), C.byref(self.launch), self.workspace.data_ptr(),
            self.workspace.numel(), nat.stream_handle(stream)))
