"""Trajectory frames in the reference's binary format, so that its offline
analyzers (analyze/read.h) read what this library writes.

Writer -- operator<<(ostream&, Box*), parallel/box.h:476-502:
  header  t, Lx, Ly as float64 (Lx = Ly = the half-width L of the box
          [-L, L)^2), nb (int32, chain length of the first swimmer), Ns, Nm
          (int32)
  then    Nm membrane beads: (x, y) float32, the unwrapped position
          r_original (C2DVector::write, shared/c2dvector.h:175-184)
          Ns swimmers: (x, y, theta) float32, x, y unwrapped
          (RepulsiveParticle::Write, shared/particle.h:759-764;
          ActiveBrownianChain::Write, :1022-1045)
Frames follow one another with no separator.

Reader -- Scene operator>> (analyze/read.h:215-270) and
SceneSet::Count_Frames (:358-398): a frame is unhealthy when it is cut
short, when t < 0 or t > 1e6, or when Nm < 0 or Nm > 1e6; reading stops at
the first frame cut short.  Ns and Nm are taken from the first header.
"""
import struct
from dataclasses import dataclass

import numpy as np

from . import abi

HEADER = struct.Struct("<dddiii")


@dataclass
class Frame:
    t: float
    Lx: float
    Ly: float
    nb: int
    x: np.ndarray        # swimmers, unwrapped
    y: np.ndarray
    theta: np.ndarray
    mx: np.ndarray       # membrane beads, unwrapped
    my: np.ndarray
    healthy: bool = True


def encode_frame(t, L, x, y, theta, mx=None, my=None, nb=1):
    """Bytes of one frame (positions already unwrapped)."""
    x = np.asarray(x, np.float32)
    mx = np.zeros(0, np.float32) if mx is None else np.asarray(mx, np.float32)
    my = np.zeros(0, np.float32) if my is None else np.asarray(my, np.float32)
    head = HEADER.pack(float(t), float(L), float(L), int(nb), len(x), len(mx))
    mem = np.stack([mx, my], 1).astype("<f4").tobytes()
    sw = np.stack([x, np.asarray(y, np.float32), np.asarray(theta, np.float32)], 1).astype("<f4").tobytes()
    return head + mem + sw


def state_frame(p, t, x, y, theta, img_x, img_y):
    """Bytes of one frame of a system's state (spp_download_state arrays):
    membrane beads (the first n_rings x ring_size particles of a bead model)
    write (x, y), the others (x, y, theta); positions are unwrapped with the
    image counters."""
    L = float(p.L)
    xu = (np.asarray(x, np.float64) + 2.0 * L * np.asarray(img_x, np.float64)).astype(np.float32)
    yu = (np.asarray(y, np.float64) + 2.0 * L * np.asarray(img_y, np.float64)).astype(np.float32)
    nm = p.n_rings * p.ring_size if p.model == abi.MODEL_BEADS else 0
    # the header's nb is the first swimmer's (particle[Nm].nb, parallel/box.h:485)
    nb = p.chain_beads if p.model == abi.MODEL_BEADS and p.chain_beads > 1 else 1
    return encode_frame(t, L, xu[nm:], yu[nm:], np.asarray(theta, np.float32)[nm:], xu[:nm], yu[:nm],
                        nb=nb)


def write_system_frame(f, system, t=None):
    """Appends the system's current state to the open binary file f."""
    x, y, th, ix, iy = system.download()
    obs = system.observables()
    f.write(state_frame(system.params, obs.t if t is None else t, x, y, th, ix, iy))


def read_frames(data):
    """Frames of a .bin file (path or bytes), with the reference reader's
    health rules; a frame cut short ends the list and is not returned."""
    if not isinstance(data, (bytes, bytearray)):
        with open(data, "rb") as fh:
            data = fh.read()
    frames = []
    if len(data) < HEADER.size:
        return frames
    _, _, _, _, Ns, Nm = HEADER.unpack_from(data, 0)
    size = HEADER.size + 8 * Nm + 12 * Ns
    off = 0
    while off + HEADER.size <= len(data):
        t, Lx, Ly, nb, _, nm_field = HEADER.unpack_from(data, off)
        if off + size > len(data):
            break
        body = off + HEADER.size
        mem = np.frombuffer(data, "<f4", 2 * Nm, body).reshape(Nm, 2)
        sw = np.frombuffer(data, "<f4", 3 * Ns, body + 8 * Nm).reshape(Ns, 3)
        healthy = not (t < 0 or t > 1e6) and not (nm_field < 0 or nm_field > 1000000)
        frames.append(Frame(t, Lx, Ly, nb, sw[:, 0].copy(), sw[:, 1].copy(), sw[:, 2].copy(),
                            mem[:, 0].copy(), mem[:, 1].copy(), healthy))
        off += size
    return frames
