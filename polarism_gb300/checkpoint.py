"""Checkpoint format 2 for the GPU-resident state
(``polarism/simulation_controller.py:736-923``, ``save_checkpoint`` / ``load_checkpoint``).

Besides the field and the reservoir, a run on the GPU keeps three things in device memory that
format 2 stores: the steady-state reference (``steady_density``, ``steady_norm``) and the stop
times of the device monitor, and the FP64 accumulator sums (``accumulators/<name>``).
:func:`capture` collects them from an :class:`~polarism_gb300.engine.RK4Engine` into the
format's entries, :func:`restore` puts them back, and :func:`save` / :func:`load` write and read
the entries: as the reference's HDF5 file when ``h5py`` is installed and the path ends in
``.h5`` (attributes, groups and datasets named as ``save_checkpoint`` names them), otherwise as
an ``.npz`` archive whose keys are the same names (``attrs/step``, ``reservoir/nR``,
``accumulators/g2/sum_density``, ...).

Array shapes follow the reference's public state: the member axis only when ``batched``, the
component axis only for two-component fields (``polarism/results/accumulators.py:55``).
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

VERSION = 2

#: accumulator name -> (engine kind, dataset name) pairs (``accumulators.py:94-172``)
ACCUMULATORS = {
    "g2": (("rho", "sum_density"), ("rho2", "sum_density_squared")),
    "momentum-distribution": (("k", "sum_k"),),
}

#: reservoir type -> the reservoir's ``state_names``, the order of its fields in the engine
#: (``single_reservoir.py:24``, ``double_reservoir.py:24``, ``quadratic_double_reservoir.py:43``,
#: ``no_reservoir.py:12``)
STATE_NAMES = {
    "single": ("nR",),
    "double": ("nA", "nI"),
    "quadratic-double": ("nR", "nI"),
    "none": (),
}


def reservoir_fields(ckpt):
    """The checkpoint's reservoir fields in the engine's order.

    A file stores them by name and HDF5 lists a group's members alphabetically, so the order
    comes from the reservoir type's ``state_names``; as ``load_checkpoint`` does
    (``simulation_controller.py:858-861``), a name set other than that type's is an error."""
    stored = ckpt["reservoir"]
    kind = str(ckpt["attrs"].get("reservoir_type", ""))
    names = STATE_NAMES.get(kind)
    if names is None:  # a reservoir this library does not model: keep the stored order
        return [np.asarray(v) for v in stored.values()]
    if set(stored) != set(names):
        raise ValueError(f"checkpoint reservoir names mismatch: {sorted(stored)} stored, "
                         f"{list(names)} expected for reservoir type {kind!r}")
    return [np.asarray(stored[n]) for n in names]


def _public(array, batched, components):
    """(B, C, ...) engine layout -> the reference's public shape."""
    out = np.asarray(array)
    if components == 1:
        out = out[:, 0]
    return out if batched else out[0]


def _engine_layout(array, batched, components):
    out = np.asarray(array)
    if not batched:
        out = out[None]
    if components == 1:
        out = out[:, None]
    return out


def capture(engine, *, step, t0, dt, reservoir_names, reservoir_type, batched=True, components=1,
            config_json="{}", steady_last_step=-1, accumulators=None, field_k=None,
            step_controller=None):
    """Format-2 entries of the engine's state after ``step`` steps.

    ``accumulators`` maps a name of :data:`ACCUMULATORS` to ``{"t_first": .., "t_last": ..}``
    (the host-side sampling metadata); sums and sample counts come from the device."""
    psi, res = engine.get_state()
    attrs = {
        "checkpoint_version": VERSION, "polarism_version": "polarism_gb300",
        "step": int(step), "t": float(t0 + step * dt), "t0": float(t0), "dt": float(dt),
        "ndim": 2, "shape": np.asarray([engine.ny, engine.nx]), "components": int(components),
        "batched": bool(batched), "reservoir_type": str(reservoir_type),
        "config_json": config_json, "steady_last_step": int(steady_last_step),
    }
    density, norms, stops = engine.steady_export()
    attrs["stop_time"] = np.where(stops >= 0, t0 + stops * dt, np.nan)
    data = {"field": np.asarray(psi)}  # (B, C, ny, nx), as the reference's state.field
    if field_k is not None:
        data["field_k"] = np.asarray(field_k)
    if density is not None:
        attrs["steady_norm"] = norms
        data["steady_density"] = density if batched else density[0]
    fields = res if np.ndim(res) == 5 else np.asarray(res)[None]
    reservoir = {name: np.asarray(fields[i]) for i, name in enumerate(reservoir_names)}
    accumulated = {}
    for name, meta in (accumulators or {}).items():
        entry = {"t_first": meta.get("t_first"), "t_last": meta.get("t_last")}
        for kind, key in ACCUMULATORS[name]:
            sums, samples = engine.accumulator_sums(kind)
            entry[key] = _public(sums, batched, components)
            entry["samples"] = int(samples)
        accumulated[name] = entry
    return {"attrs": attrs, "data": data, "reservoir": reservoir, "accumulators": accumulated,
            "step_controller": dict(step_controller) if step_controller is not None else None}


def restore(engine, ckpt):
    """Load a :func:`capture` / :func:`load` result into ``engine``; returns the step."""
    attrs = ckpt["attrs"]
    if int(attrs["checkpoint_version"]) != VERSION:
        raise ValueError(f"checkpoint format v{attrs['checkpoint_version']} is not supported; "
                         f"supported: {VERSION}")
    batched = bool(attrs["batched"])
    components = int(attrs["components"])
    step, t, t0, dt = int(attrs["step"]), float(attrs["t"]), float(attrs["t0"]), float(attrs["dt"])
    if step < 0 or not math.isclose(t, t0 + step * dt, rel_tol=0.0, abs_tol=1e-9 * max(1.0, abs(t))):
        raise ValueError("checkpoint time and step mismatch")
    field = np.asarray(ckpt["data"]["field"])
    fields = reservoir_fields(ckpt)
    res = fields[0] if len(fields) == 1 else np.stack(fields) if fields else None
    engine.set_state(np.ascontiguousarray(field, dtype=engine.complex),
                     np.ascontiguousarray(res, dtype=engine.real) if fields else None)
    stop_time = np.asarray(attrs.get("stop_time", np.full(engine.members, np.nan)), dtype=float)
    stops = np.where(np.isfinite(stop_time), np.round((stop_time - t0) / dt), -1).astype(np.int64)
    density = ckpt["data"].get("steady_density")
    if density is not None:
        density = np.asarray(density).reshape(engine.members, engine.ny, engine.nx)
    engine.steady_import(density, attrs.get("steady_norm"), stops)
    for name, entry in ckpt["accumulators"].items():
        for kind, key in ACCUMULATORS[name]:
            engine.accumulator_load(kind, _engine_layout(entry[key], batched, components),
                                    int(entry["samples"]))
    return step


# ------------------------------------------------------------------------------ files
def _flatten(ckpt):
    flat = {f"attrs/{k}": np.asarray(v) for k, v in ckpt["attrs"].items()}
    flat.update({k: np.asarray(v) for k, v in ckpt["data"].items()})
    flat.update({f"reservoir/{k}": np.asarray(v) for k, v in ckpt["reservoir"].items()})
    flat["attrs/reservoir_names"] = np.asarray(list(ckpt["reservoir"]))
    for name, entry in ckpt["accumulators"].items():
        for key, value in entry.items():
            flat[f"accumulators/{name}/{key}"] = np.asarray(np.nan if value is None else value)
    if ckpt.get("step_controller") is not None:
        for key, value in ckpt["step_controller"].items():
            flat[f"step_controller/{key}"] = np.asarray(value)
    return flat


def _unflatten(flat):
    ckpt = {"attrs": {}, "data": {}, "reservoir": {}, "accumulators": {}, "step_controller": None}
    names = [str(n) for n in flat.pop("attrs/reservoir_names", [])]
    for key, value in flat.items():
        value = value[()] if np.ndim(value) == 0 else value
        if key.startswith("attrs/"):
            ckpt["attrs"][key[6:]] = value
        elif key.startswith("reservoir/"):
            ckpt["reservoir"][key[10:]] = value
        elif key.startswith("accumulators/"):
            _, name, item = key.split("/", 2)
            entry = ckpt["accumulators"].setdefault(name, {})
            if item in ("t_first", "t_last"):
                value = None if np.isnan(value) else float(value)
            entry[item] = value
        elif key.startswith("step_controller/"):
            ckpt["step_controller"] = ckpt["step_controller"] or {}
            ckpt["step_controller"][key[16:]] = value
        else:
            ckpt["data"][key] = value
    if names:
        ckpt["reservoir"] = {n: ckpt["reservoir"][n] for n in names}
    for key in ("config_json", "reservoir_type", "polarism_version"):
        if key in ckpt["attrs"]:
            ckpt["attrs"][key] = str(ckpt["attrs"][key])
    return ckpt


def save(path, ckpt):
    """Write ``ckpt`` (a :func:`capture` result) to ``path``."""
    path = Path(path)
    if path.suffix == ".h5":
        import h5py  # the reference's own format; h5py is a dependency of the reference

        with h5py.File(path, "w") as h5:
            for key, value in ckpt["attrs"].items():
                h5.attrs[key] = value
            for key, value in ckpt["data"].items():
                h5.create_dataset(key, data=value)
            group = h5.create_group("reservoir")
            for key, value in ckpt["reservoir"].items():
                group.create_dataset(key, data=value)
            if ckpt["accumulators"]:
                accumulated = h5.create_group("accumulators")
                for name, entry in ckpt["accumulators"].items():
                    saved = accumulated.create_group(name)
                    for key, value in entry.items():
                        if key in ("samples", "t_first", "t_last"):
                            saved.attrs[key] = np.nan if value is None else value
                        else:
                            saved.create_dataset(key, data=value)
            if ckpt.get("step_controller") is not None:
                h5.create_group("step_controller").attrs.update(ckpt["step_controller"])
        return path
    np.savez(path, **_flatten(ckpt))
    return path if path.suffix == ".npz" else path.with_name(path.name + ".npz")


def load(path):
    """Read a checkpoint written by :func:`save` or by the reference (``.h5``)."""
    path = Path(path)
    if path.suffix == ".h5":
        import h5py

        with h5py.File(path, "r") as h5:
            flat = {f"attrs/{k}": np.asarray(v) for k, v in h5.attrs.items()}
            for key in h5:
                if key == "reservoir":
                    flat.update({f"reservoir/{n}": h5["reservoir"][n][()] for n in h5["reservoir"]})
                    flat["attrs/reservoir_names"] = np.asarray(list(h5["reservoir"]))
                elif key == "accumulators":
                    for name, group in h5["accumulators"].items():
                        for a, v in group.attrs.items():
                            flat[f"accumulators/{name}/{a}"] = np.asarray(v)
                        for d in group:
                            flat[f"accumulators/{name}/{d}"] = group[d][()]
                elif key == "step_controller":
                    for a, v in h5["step_controller"].attrs.items():
                        flat[f"step_controller/{a}"] = np.asarray(v)
                else:
                    flat[key] = h5[key][()]
        return _unflatten(flat)
    with np.load(path, allow_pickle=False) as data:
        return _unflatten({k: data[k] for k in data.files})


def config_json(cfg) -> str:
    """JSON of a host-mirror config, as ``save_checkpoint`` stores ``asdict(cfg)``."""
    from dataclasses import asdict, is_dataclass

    return json.dumps(asdict(cfg) if is_dataclass(cfg) else dict(cfg))
