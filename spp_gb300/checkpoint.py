"""Bit-exact checkpoint and resume of a system.

Replaces the reference's restart path -- a saved frame read back by
operator>>(istream&, Box*) (parallel/box.h:505-524) and re-placed by
Positioning_Particles (:155-218) -- which cannot continue the same noise,
since the GSL generator state is not saved.  A checkpoint here holds the
parameters, the wrapped positions with their box-crossing counters, the
headings, the Philox step counter and, for run-and-tumble swimmers, the
tumble state of every particle: the noise of a step is a function of (seed,
system, particle, step), so a resumed run continues bit for bit.
File: a numpy .npz archive (params as the raw SppParams bytes); format 2
adds the tumble state (format 1 files, without it, still load)."""
import ctypes as C

import numpy as np

from . import abi
from .system import Snapshot, System

FORMAT = 2


def save(path, system: System, step=None):
    """Writes the system's parameters and state; step = the Philox step
    counter of the state (default: the steps the system has taken since its
    upload plus the upload's step0)."""
    x, y, th, ix, iy = system.download()
    if step is None:
        step = system.step0 + int(system.observables().step)
    raw = bytes(C.string_at(C.addressof(system.params), C.sizeof(system.params)))
    extra = {}
    tumble = system.download_tumble()
    if tumble is not None:
        extra["tumble"] = tumble
    np.savez(path, format=FORMAT, params=np.frombuffer(raw, np.uint8), x=x, y=y, theta=th, img_x=ix,
             img_y=iy, step=np.int64(step), **extra)


def load(path):
    """(SppParams, Snapshot) of a checkpoint file."""
    with np.load(path) as z:
        if int(z["format"]) not in (1, FORMAT):
            raise ValueError(f"unknown checkpoint format {int(z['format'])}")
        raw = z["params"].tobytes()
        n = C.sizeof(abi.SppParams)
        # SppParams only grows at its end and starts with its own size: a
        # shorter record of an earlier layout reads with the later fields 0
        # (chain_beads 0 = single beads, rot_noise 0 = Gaussian noise)
        if len(raw) < 4 or len(raw) > n or int.from_bytes(raw[:4], "little") != len(raw):
            raise ValueError("checkpoint was written with a different SppParams layout")
        p = abi.SppParams()
        C.memmove(C.addressof(p), raw, len(raw))
        p.struct_size = n
        snap = Snapshot(z["x"].copy(), z["y"].copy(), z["theta"].copy(), z["img_x"].copy(), z["img_y"].copy(),
                        int(z["step"]), z["tumble"].copy() if "tumble" in z.files else None)
    return p, snap


def resume(path) -> System:
    """A new system holding the checkpointed state, ready to continue."""
    p, snap = load(path)
    s = System(p)
    s.upload(snap.x, snap.y, snap.theta, step0=snap.step, img_x=snap.img_x, img_y=snap.img_y)
    if snap.tumble is not None:
        s.upload_tumble(snap.tumble)
    return s
