"""Launch-shape autotuner with a persistent table keyed by (model, N, density).

``autotune`` runs ``spp_autotune`` (include/spp.h) on a given state: it times
every candidate shape -- threads per particle in the neighbour sums
(``gather_lanes`` 1 or 4; ABP, continuous and single-bead bead models) and the Verlet skin
(0.5, 1, 1.5, 2 x the requested one) -- and returns the parameters with the
fastest written in.  ``tuned_params`` looks the system up in a ``TuneTable``
first and measures only on a miss, on a seeded uniform state of the same
size and density unless a state is given.

The reference fixes these from compile-time globals (shared/parameters.h:
80-99) for every system.  Here the best shape depends on the system: four
lanes per particle pay when the system is too small to fill the GPU or its
lists are long (flocks, dense clusters); a wider skin pays when rebuilds
cost more than the longer lists.  The skin does not change the trajectory
(lists are summed in particle-id order); the lane count fixes the order of
the neighbour additions and so is part of the result, like any parameter.

Table keys bucket N by octave and the density by half octave; the model,
integrator, force law, alignment mode, boundary, the requested skin, the
distance travelled per step (v0 dt) and which shapes were tuned are part of
the key as well.
"""
import ctypes as C
import json
import math
import os
from pathlib import Path

import numpy as np

from . import abi, configs

DEFAULT_TABLE = Path(os.environ.get("SPP_TUNE_TABLE",
                                    Path.home() / ".cache" / "spp_gb300" / "tune.json"))


def density(p) -> float:
    """Particles per unit area of the box [-L, L)^2."""
    return p.n / (2.0 * p.L) ** 2


def table_key(p) -> str:
    n_oct = int(round(math.log2(max(p.n, 1))))
    rho_half_oct = round(2.0 * math.log2(density(p))) / 2.0
    return (f"model{p.model}-int{p.integrator}-law{p.force_law}-align{p.align_mode}-"
            f"bound{p.boundary}-n2^{n_oct}-rho2^{rho_half_oct:+.1f}-"
            f"skin{p.skin:.4g}-step{p.v0 * p.dt:.4g}")


class TuneTable:
    """Chosen shapes by table key, kept in a JSON file."""

    def __init__(self, path=None):
        self.path = Path(path) if path is not None else DEFAULT_TABLE
        self.entries = {}
        if self.path.exists():
            self.entries = json.loads(self.path.read_text())

    def get(self, key):
        return self.entries.get(key)

    def put(self, key, entry):
        self.entries[key] = entry
        self.path.parent.mkdir(parents=True, exist_ok=True)
        tmp = self.path.with_suffix(self.path.suffix + ".tmp")
        tmp.write_text(json.dumps(self.entries, indent=1, sort_keys=True))
        tmp.replace(self.path)


def report_rows(rep: abi.SppTuneReport):
    """The candidates of a report as dicts, in the order tried."""
    rows = []
    for i in range(rep.n_candidates):
        c = rep.c[i]
        rows.append({"gather_lanes": int(c.gather_lanes), "skin": float(c.skin),
                     "ms_per_step": float(c.ms_per_step), "late_rebuilds": int(c.late_rebuilds),
                     "status": int(c.status), "chosen": i == rep.best})
    return rows


def autotune(p, x, y, theta, trial_steps=200, what=abi.TUNE_LANES | abi.TUNE_SKIN):
    """Times the candidate shapes on the device; returns (tuned params, rows)."""
    q = p.copy()
    if q.struct_size == 0:
        q.struct_size = C.sizeof(abi.SppParams)
    f32 = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, theta)]
    for a in f32:
        if a.shape != (q.n,):
            raise ValueError(f"state arrays must hold n = {q.n} values")
    rep = abi.SppTuneReport()
    ptr = [a.ctypes.data_as(C.POINTER(C.c_float)) for a in f32]
    abi.check(abi.lib().spp_autotune(C.byref(q), ptr[0], ptr[1], ptr[2], int(trial_steps), int(what),
                                     C.byref(rep)), "spp_autotune")
    return q, report_rows(rep)


def tuned_params(p, table=None, state=None, trial_steps=200, what=abi.TUNE_LANES | abi.TUNE_SKIN,
                 seed=0, measure=autotune):
    """p with the table's shape for its key, measured (and stored) on a miss.

    state: (x, y, theta) to time on; by default a seeded uniform state of p's
    size in p's box.  measure: the timing function (``autotune``)."""
    table = table if table is not None else TuneTable()
    key = f"{table_key(p)}-tune{int(what)}"
    hit = table.get(key)
    if hit is None:
        if state is None:
            state = configs.random_state(p.n, p.L, seed=seed)
        q, rows = measure(p, *state, trial_steps=trial_steps, what=what)
        best = next(r for r in rows if r["chosen"])
        hit = {"gather_lanes": int(q.gather_lanes), "skin_factor": float(q.skin) / float(p.skin),
               "ms_per_step": best["ms_per_step"], "candidates": rows}
        table.put(key, hit)
    return p.replace(gather_lanes=int(hit["gather_lanes"]), skin=float(p.skin) * float(hit["skin_factor"]))
