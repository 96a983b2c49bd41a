"""Host-side mirror of the reference's Box interface over the C ABI.

``System`` is a thin owner of one ``SppSystem*``.  ``Box`` keeps the method
names of the reference's Box (parallel/box.h:15-58, serial/box.h:15-61) so
that driver code written against the reference keeps its shape:

    reference                              here
    ---------------------------------------------------------------------
    Box(Lx, Ly, phi) + Init(node, rho)     Box(params); Init(x, y, theta)
    Sync()                                 Sync()           (re-bin + list)
    Update_Cells / Update_Neighbor_List    Update_Cells()   (same rebuild)
    One_Step()                             One_Step()
    Multi_Step(steps)                      Multi_Step(steps)
    Multi_Step(steps, interval)            Multi_Step(steps, interval)
    Save(sv) / Load(sv)                    Save() -> Snapshot / Load(snap)
    Save_Polarization(os)                  Save_Polarization(stream)
    Compute_Polarization()                 Compute_Polarization()
    operator<<(os, box)                    Write(stream)   (.bin frame)

Errors surface as ``SppError`` carrying the ABI status, where the reference
prints and exits (shared/cell.h:45-49, parallel/box.h:224-228).
"""
import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import abi


class System:
    def __init__(self, params: abi.SppParams):
        self.params = params.copy()
        if self.params.struct_size == 0:
            self.params.struct_size = C.sizeof(abi.SppParams)
        self._h = C.c_void_p()
        abi.check(abi.lib().spp_create(C.byref(self.params), C.byref(self._h)), "spp_create")
        self.n = int(self.params.n)
        self.step0 = 0

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            abi.lib().spp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, x, y, theta, step0=0, img_x=None, img_y=None):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        th = np.ascontiguousarray(theta, np.float32)
        ix = None if img_x is None else np.ascontiguousarray(img_x, np.int32)
        iy = None if img_y is None else np.ascontiguousarray(img_y, np.int32)
        abi.check(abi.lib().spp_upload_state(self._h, abi.fptr(x), abi.fptr(y), abi.fptr(th),
                                             abi.iptr(ix), abi.iptr(iy), self.n, int(step0)),
                  "spp_upload_state")
        self.step0 = int(step0)

    def download(self, out=None):
        """(x, y, theta, img_x, img_y) in particle-id order; out = five arrays
        (float32, float32, float32, int32, int32, length n) to fill instead of
        new ones, e.g. pinned host buffers."""
        n = self.n
        if out is not None:
            x, y, th, ix, iy = out
            for a, dt in zip(out, (np.float32, np.float32, np.float32, np.int32, np.int32)):
                if a.dtype != dt or a.shape != (n,) or not a.flags.c_contiguous:
                    raise ValueError("download buffers must be contiguous arrays of length n")
        else:
            x = np.empty(n, np.float32)
            y = np.empty(n, np.float32)
            th = np.empty(n, np.float32)
            ix = np.empty(n, np.int32)
            iy = np.empty(n, np.int32)
        abi.check(abi.lib().spp_download_state(self._h, abi.fptr(x), abi.fptr(y), abi.fptr(th),
                                               abi.iptr(ix), abi.iptr(iy), n), "spp_download_state")
        return x, y, th, ix, iy

    @property
    def has_tumble(self):
        """Run-and-tumble swimmers carry a per-particle tumble state."""
        return int(self.params.rot_noise) == abi.NOISE_TUMBLE

    def download_tumble(self):
        """Run-and-tumble state per particle id (int32: 0 running, +-c in the
        c-th step of a tumble), or None without run and tumble."""
        if not self.has_tumble:
            return None
        st = np.empty(self.n, np.int32)
        abi.check(abi.lib().spp_download_tumble(self._h, abi.iptr(st), self.n), "spp_download_tumble")
        return st

    def upload_tumble(self, state):
        st = np.ascontiguousarray(state, np.int32)
        abi.check(abi.lib().spp_upload_tumble(self._h, abi.iptr(st), self.n), "spp_upload_tumble")

    def step(self, nsteps):
        abi.check(abi.lib().spp_step(self._h, int(nsteps)), "spp_step")

    def sync(self):
        abi.check(abi.lib().spp_sync(self._h), "spp_sync")

    def observables(self) -> abi.SppObservables:
        o = abi.SppObservables()
        abi.check(abi.lib().spp_observables(self._h, C.byref(o)), "spp_observables")
        return o

    def pairs(self, r, cap=None):
        """Unique pairs (i < j, particle ids) within r under the kernels'
        FP32 predicate, sorted as int64 keys i << 32 | j."""
        cap = cap if cap is not None else max(16, 8 * self.n)
        pi = np.empty(cap, np.int32)
        pj = np.empty(cap, np.int32)
        cnt = C.c_int64()
        abi.check(abi.lib().spp_pairs(self._h, float(r), abi.iptr(pi), abi.iptr(pj), cap,
                                      C.byref(cnt)), "spp_pairs")
        if cnt.value > cap:
            return self.pairs(r, cap=int(cnt.value))
        a = np.minimum(pi[:cnt.value], pj[:cnt.value]).astype(np.int64)
        b = np.maximum(pi[:cnt.value], pj[:cnt.value]).astype(np.int64)
        return np.sort(a * (1 << 32) + b)

    def cells(self, D, rule=abi.BIN_GEOMETRIC):
        cx = np.empty(self.n, np.int32)
        cy = np.empty(self.n, np.int32)
        abi.check(abi.lib().spp_cells(self._h, int(D), int(rule), abi.iptr(cx), abi.iptr(cy),
                                      self.n), "spp_cells")
        return cx, cy

    def kernel_launches(self):
        return int(abi.lib().spp_kernel_launches(self._h))

    def stream(self):
        return abi.lib().spp_stream(self._h)

    # ---- tangent-space Lyapunov spectrum (LyapunovBox counterpart) ----
    def lyap_init(self, k, seed=3):
        self._lyap_k = int(k)
        abi.check(abi.lib().spp_lyap_init(self._h, int(k), int(seed)), "spp_lyap_init")

    def lyap_set_vectors(self, v):
        v = np.ascontiguousarray(v, np.float32)
        abi.check(abi.lib().spp_lyap_set_vectors(self._h, abi.fptr(v), self._lyap_k),
                  "spp_lyap_set_vectors")

    def lyap_step(self, nsteps, renorm_every=10):
        abi.check(abi.lib().spp_lyap_step(self._h, int(nsteps), int(renorm_every)), "spp_lyap_step")

    def lyap_exponents(self):
        k = self._lyap_k
        lam = (C.c_double * k)()
        T = C.c_double()
        abi.check(abi.lib().spp_lyap_exponents(self._h, lam, k, C.byref(T)), "spp_lyap_exponents")
        return np.array(lam[:]), T.value

    def lyap_vectors(self):
        k = self._lyap_k
        v = np.empty(k * 3 * self.n, np.float32)
        abi.check(abi.lib().spp_lyap_vectors(self._h, abi.fptr(v), k), "spp_lyap_vectors")
        return v.reshape(k, 3, self.n)

    def time_steps(self, nsteps):
        """spp_step(nsteps) timed with CUDA events on the launching stream (ms)."""
        ms = C.c_double()
        abi.check(abi.lib().spp_time_steps(self._h, int(nsteps), C.byref(ms)), "spp_time_steps")
        return ms.value

    def polarization_series(self, nframes, every=1):
        """Advances nframes x every steps, P after every `every` steps
        (returns p, px, py as float64 arrays)."""
        p = np.empty(nframes, np.float64)
        px = np.empty(nframes, np.float64)
        py = np.empty(nframes, np.float64)
        D = lambda a: a.ctypes.data_as(abi._D)
        abi.check(abi.lib().spp_polarization_series(self._h, int(nframes), int(every), D(p), D(px), D(py)),
                  "spp_polarization_series")
        return p, px, py

    def radial_distribution(self, r_max, nbins):
        """Ordered-pair counts of minimum-image distances < r_max in nbins bins."""
        out = np.zeros(nbins, np.uint64)
        abi.check(abi.lib().spp_radial_distribution(self._h, float(r_max), int(nbins),
                                                     out.ctypes.data_as(abi._U64)), "spp_radial_distribution")
        return out

    def pair_distribution(self, lx, ly, gx, gy):
        """Body-frame pair counts [gx][gy] (the reference's Pair_Distribution)."""
        out = np.zeros(gx * gy, np.uint64)
        abi.check(abi.lib().spp_pair_distribution(self._h, float(lx), float(ly), int(gx), int(gy),
                                                   out.ctypes.data_as(abi._U64)), "spp_pair_distribution")
        return out.reshape(gx, gy)

    def ring_shapes(self):
        """Per ring vesicle: shape of the membrane (mb_*) and of its swimmers
        (sw_*) -- centre of mass, gyration tensor, eigenvalues, Rg, asphericity
        (Box::Compute_All_Variables, parallel/beadbox.h:325-434).  Returns a
        dict of arrays."""
        nr = int(self.params.n_rings)
        out = (abi.SppRingShape * nr)()
        abi.check(abi.lib().spp_ring_shapes(self._h, out, nr), "spp_ring_shapes")
        return {name: np.array([getattr(o, name) for o in out]) for name, _ in abi.SppRingShape._fields_}

    def ring_motion_mark(self):
        """Save the current frame (positions and headings) for ring_motion
        (Save_Particles_Positions, parallel/beadbox.h:315-322)."""
        abi.check(abi.lib().spp_ring_motion_mark(self._h), "spp_ring_motion_mark")

    def ring_motion(self):
        """Per ring vesicle, the motion since the marked frame: centre-of-mass
        velocities, angular momenta, rotation rates and the swimmers' mean spin
        (Box::Compute_All_Variables, parallel/beadbox.h:325-434); marks the
        current frame.  Returns a dict of arrays."""
        nr = int(self.params.n_rings)
        out = (abi.SppRingMotion * nr)()
        abi.check(abi.lib().spp_ring_motion(self._h, out, nr), "spp_ring_motion")
        return {name: np.array([getattr(o, name) for o in out]) for name, _ in abi.SppRingMotion._fields_}

    def profile(self, nsteps):
        pr = abi.SppProfile()
        abi.check(abi.lib().spp_profile(self._h, int(nsteps), C.byref(pr)), "spp_profile")
        return pr


@dataclass
class Snapshot:
    """State_Hyper_Vector counterpart (shared/state-hyper-vector.h:6-41): the
    positions, headings and the Philox step counter, which makes a reload
    reproduce the same noise (the reference copies the GSL state instead,
    :169-177)."""
    x: np.ndarray
    y: np.ndarray
    theta: np.ndarray
    img_x: np.ndarray
    img_y: np.ndarray
    step: int
    tumble: Optional[np.ndarray] = None   # run-and-tumble state (RTPChain), if any


class Box:
    """Reference-shaped driver interface (parallel/box.h:15-58)."""

    def __init__(self, params: abi.SppParams):
        self.params = params.copy()
        self.system = System(self.params)
        self.t = 0.0
        self.polarization = 0.0
        self._step0 = 0

    @property
    def N(self):
        return self.system.n

    def Init(self, x, y, theta, t=0.0):
        """Box::Init / Positioning_Particles: place particles, bin, build lists."""
        step0 = int(round(t / self.params.dt))
        self.system.upload(x, y, theta, step0=step0)
        self._step0 = step0
        self.t = t

    def Sync(self):
        """Re-bin and rebuild the neighbour list from the current state."""
        s = self.Save()
        self.Load(s)

    Update_Cells = Sync
    Update_Neighbor_List = Sync

    def One_Step(self):
        self.system.step(1)
        self.t += self.params.dt

    def Multi_Step(self, steps, interval=None):
        """Box::Multi_Step(steps) / Multi_Step(steps, interval): the cell
        update interval is irrelevant here (rebuilds are displacement-
        triggered on the device), so both forms advance `steps` steps."""
        self.system.step(int(steps))
        self.t += self.params.dt * int(steps)

    def Save(self) -> Snapshot:
        x, y, th, ix, iy = self.system.download()
        o = self.system.observables()
        return Snapshot(x, y, th, ix, iy, self._step0 + int(o.step), self.system.download_tumble())

    def Load(self, snap: Snapshot):
        self.system.upload(snap.x, snap.y, snap.theta, step0=snap.step, img_x=snap.img_x,
                           img_y=snap.img_y)
        if snap.tumble is not None:
            self.system.upload_tumble(snap.tumble)
        self._step0 = snap.step
        self.t = snap.step * self.params.dt

    def Compute_Polarization(self):
        self.polarization = self.system.observables().polarization
        return self.polarization

    def Save_Polarization(self, os):
        """Box::Save_Polarization (parallel/box.h:467-473): 't<TAB>P' per line."""
        os.write(f"{self.t}\t{self.Compute_Polarization()}\n")

    def Write(self, os):
        """operator<<(ostream&, Box*) (parallel/box.h:476-502): one binary frame
        in the reference's format (spp_gb300.binfile): header t, Lx, Ly, nb,
        Ns, Nm, then membrane beads (x, y) and swimmers (x, y, theta) as
        float32, positions unwrapped (r_original)."""
        from . import binfile
        x, y, th, ix, iy = self.system.download()
        os.write(binfile.state_frame(self.params, self.t, x, y, th, ix, iy))


class Batch:
    """Many independent Vicsek-family systems in one set of launches
    (replaces the serial/mpi-main.cpp:157-176 task farm)."""

    def __init__(self, systems):
        self.params = [q.copy() for q in systems]
        for q in self.params:
            if q.struct_size == 0:
                q.struct_size = C.sizeof(abi.SppParams)
        arr = (abi.SppParams * len(self.params))(*self.params)
        self._h = C.c_void_p()
        abi.check(abi.lib().spp_batch_create(arr, len(self.params), C.byref(self._h)),
                  "spp_batch_create")
        self.n_sys = len(self.params)
        self.sizes = np.array([q.n for q in self.params], np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])
        self.n_total = int(self.offsets[-1])

    def close(self):
        if self._h:
            abi.lib().spp_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_windows(self, window, stationary_from, max_steps):
        abi.check(abi.lib().spp_batch_set_windows(self._h, int(window), int(stationary_from),
                                                  int(max_steps)), "spp_batch_set_windows")

    def upload(self, x, y, theta):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        th = np.ascontiguousarray(theta, np.float32)
        abi.check(abi.lib().spp_batch_upload(self._h, abi.fptr(x), abi.fptr(y), abi.fptr(th),
                                             self.n_total), "spp_batch_upload")

    def step(self, nsteps):
        abi.check(abi.lib().spp_batch_step(self._h, int(nsteps)), "spp_batch_step")

    def time_steps(self, nsteps):
        ms = C.c_double()
        abi.check(abi.lib().spp_batch_time_steps(self._h, int(nsteps), C.byref(ms)),
                  "spp_batch_time_steps")
        return ms.value

    def poll(self):
        out = (abi.SppSweepStats * self.n_sys)()
        abi.check(abi.lib().spp_batch_poll(self._h, out, self.n_sys), "spp_batch_poll")
        return list(out)

    def retire(self, systems):
        """Stops the given systems; they leave the launch space at the next step."""
        idx = np.ascontiguousarray(systems, np.int32)
        abi.check(abi.lib().spp_batch_retire(self._h, abi.iptr(idx), len(idx)), "spp_batch_retire")

    def resume(self, systems):
        """Restarts retired systems (not those that reached max_steps) where they stopped."""
        idx = np.ascontiguousarray(systems, np.int32)
        abi.check(abi.lib().spp_batch_resume(self._h, abi.iptr(idx), len(idx)), "spp_batch_resume")

    def download(self):
        n = self.n_total
        x = np.empty(n, np.float32)
        y = np.empty(n, np.float32)
        th = np.empty(n, np.float32)
        ix = np.empty(n, np.int32)
        iy = np.empty(n, np.int32)
        abi.check(abi.lib().spp_batch_download(self._h, abi.fptr(x), abi.fptr(y), abi.fptr(th),
                                               abi.iptr(ix), abi.iptr(iy), n), "spp_batch_download")
        return x, y, th, ix, iy

    def kernel_launches(self):
        return int(abi.lib().spp_batch_kernel_launches(self._h))
