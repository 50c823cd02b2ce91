"""Result files and full-population checkpoints of the memetic loop, with
resume (the reference saves results but cannot resume a run).

A checkpoint is one ``.npz`` archive whose keys are the dataset paths of the
reference's HDF5 result file (``spring/result.py:131-175``: ``pid``,
``settings``, ``pattern``, ``density_best`` / ``support_best``,
``density_avg`` / ``support_avg``, ``density_all`` / ``support_all``,
``stats/<group>/<entry>``, ``process/generation``,
``process/totgenerations``, ``process/proc_id``), plus a ``resume/`` group
with what an exact continuation needs: every individual's error metrics, the
generator state of the crossover draws, the loop's counters and the solver's
and loop's settings.  (HDF5 itself needs ``h5py``, which this environment
does not have; the layout is kept so that a converter is a loop over keys.)

Resuming rebuilds the solver from the saved input pattern and settings,
uploads the population, restores the generator, and continues: the
generations after the checkpoint are bit-identical to those of the
uninterrupted run.
"""
from __future__ import annotations

import dataclasses
import json
import os

import numpy as np

from .memetic import MemeticRun, MemeticSettings
from .phase_retrieval import Reconstruction, Solver

_METRICS = ("error", "error_real", "error_fourier", "reality", "modulesum", "complexsum", "symmetry")


def save_checkpoint(path, run: MemeticRun, pid=(0,), metadata=None):
    """Writes the result layout plus the resume state of `run` (after
    ``run.start()`` or any ``run.step()``) to `path` (.npz), atomically."""
    sol = run.solver
    out = {
        "pid": np.asarray(pid, dtype=np.int64),
        "settings": np.frombuffer(json.dumps(dataclasses.asdict(run.s)).encode(), dtype=np.uint8),
        "pattern": np.nan_to_num(sol.intensities),
        "density_best": run.best.get_density(), "support_best": run.best.get_support(),
        "density_avg": run.avg.get_density(), "support_avg": run.avg.get_support(),
        "process/generation": np.int64(run.generation),
        "process/totgenerations": np.int64(run.s.generations),
        "process/proc_id": np.int64(os.getpid()),
        "density_all": np.stack([r.get_density() for r in run.recs]),
        "support_all": np.stack([r.get_support() for r in run.recs]),
    }
    for k1, group in run.stats.get().items():
        for k2, v in group.items():
            out[f"stats/{k1}/{k2}"] = np.asarray(v, dtype=np.float64)
    for k, v in (metadata or {}).items():
        out[f"metadata/{k}"] = np.asarray(v)
    solver_args = {"center": list(sol.center), "reality": sol.reality, "realpen": sol.realpen,
                   "use_bounds": sol.use_bounds, "seed": sol.seed, "shift": [sol.shiftmin, sol.shiftmax]}
    out["resume/solver"] = np.frombuffer(json.dumps(solver_args).encode(), dtype=np.uint8)
    out["resume/metrics"] = np.array([[getattr(r, k) for k in _METRICS] for r in run.recs], dtype=np.float64)
    out["resume/rng_state"] = np.frombuffer(sol.engine.rng_state().encode(), dtype=np.uint8)
    out["resume/replcount"] = np.int64(run.replcount)
    out["resume/history"] = np.frombuffer(json.dumps(run.history).encode(), dtype=np.uint8)
    tmp = str(path) + ".tmp.npz"
    np.savez(tmp, **out)
    os.replace(tmp, str(path))


def _json(a):
    return json.loads(bytes(np.asarray(a, dtype=np.uint8)).decode())


def load_checkpoint(path):
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def resume(path, gpus=(0,)) -> MemeticRun:
    """A MemeticRun continuing the checkpointed one exactly."""
    c = load_checkpoint(path)
    settings = MemeticSettings(**_json(c["settings"]))
    sa = _json(c["resume/solver"])
    sol = Solver(c["pattern"], center=sa["center"], reality=sa["reality"], realpen=sa["realpen"],
                 use_bounds=sa["use_bounds"], gpus=list(gpus), seed=sa["seed"])
    sol.engine.set_rng_state(bytes(c["resume/rng_state"]).decode())
    recs = []
    for i in range(c["density_all"].shape[0]):
        r = Reconstruction(c["density_all"][i], c["support_all"][i])
        for k, v in zip(_METRICS, c["resume/metrics"][i]):
            setattr(r, k, float(v))
        recs.append(r)
    run = MemeticRun(sol, recs, settings)
    sol.set_shift_param(*sa["shift"])
    run.generation = int(c["process/generation"])
    run.replcount = int(c["resume/replcount"])
    run.history = _json(c["resume/history"])
    stats = {}
    for k in c:
        if k.startswith("stats/"):
            _, k1, k2 = k.split("/")
            stats.setdefault(k1, {})[k2] = c[k].tolist()
    run.stats.set(stats)
    return run
