"""The schedule autotuner's host side.

``sg_autotune`` (native, in ``libsnapy_gb300.so``) times the stage's kernels
on a handle's own blocks and state for every tile width and both forms of
the implicit solve's finish, and keeps the fastest; the results do not
depend on the choice.  A handle in sweep mode 2 (``integration/implicit-sweep:
auto``) also times the serial and the partitioned solve, whose results agree
to rounding.  This module runs it once per configuration and keeps
the choice in a JSON cache keyed by the device, the library version, the
scheme and the blocks' shapes and physics, so a later handle of the same
configuration applies it with ``sg_set_schedule`` and launches no trials.

The cache file is ``$SNAPY_GB300_TUNE_CACHE`` if set, else
``~/.cache/snapy_gb300/schedules.json``; ``SNAPY_GB300_TUNE_CACHE=off``
keeps no file (every handle tunes).
"""
from __future__ import annotations

import ctypes
import json
import os
import tempfile
from typing import Optional

import torch

from . import _lib


def cache_path() -> Optional[str]:
    p = os.environ.get("SNAPY_GB300_TUNE_CACHE")
    if p == "off":
        return None
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "snapy_gb300",
                        "schedules.json")


def key(batch) -> str:
    """The configuration a schedule belongs to."""
    from . import build as _build
    dev = torch.cuda.get_device_name(batch.device)
    try:  # a rebuilt library may want another schedule
        st = os.stat(_build.LIB)
        ver = f"{st.st_size}:{int(st.st_mtime)}"
    except OSError:
        ver = ""
    blocks = []
    for d in batch.blocks:
        blocks.append([d["nc1"], d["nc2"], d["nc3"], int(d.get("implicit_scheme", 0)),
                       int(bool(d.get("implicit_f32"))), int(d.get("grav1", 0.0) != 0.0),
                       int(d.get("nu_iso", 0.0) > 0.0), int(bool(d.get("flux_cov", True))),
                       list(d["bc"])])
    return json.dumps([dev, ver, str(batch.dtype), batch.scheme_key,
                       getattr(batch, "sweep_mode", 0), blocks],
                      separators=(",", ":"))


def _load(path: Optional[str]) -> dict:
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: Optional[str], k: str, entry: dict) -> None:
    if not path:
        return
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load(path)
        data[k] = entry
        fd, tmp = tempfile.mkstemp(dir=os.path.dirname(path), suffix=".tmp")
        with os.fdopen(fd, "w") as f:
            json.dump(data, f)
        os.replace(tmp, path)
    except OSError:
        pass  # an unwritable cache only costs a retune


def tune(batch, reps: int = 3, use_cache: bool = True, stream=None) -> dict:
    """Pick (or recall) the batch's schedule and apply it.  Returns
    {"tj": [...], "finish": f, "stage_ms": ..., "solve_ms": ..., "sweep": 0|1,
    "cached": bool}."""
    path = cache_path() if use_cache else None
    k = key(batch)
    entry = _load(path).get(k) if path else None
    n = batch.nblock
    if entry is not None and len(entry.get("tj", [])) == n:
        tj = (ctypes.c_int32 * n)(*entry["tj"])
        _lib.check(batch.L.sg_set_schedule(batch.h, tj, int(entry["finish"])),
                   "sg_set_schedule")
        if getattr(batch, "sweep_mode", 0) == 2:
            _lib.check(batch.L.sg_set_sweep(batch.h, 1 if entry.get("sweep") else 0),
                       "sg_set_sweep")
        return dict(entry, cached=True)
    tj = (ctypes.c_int32 * n)()
    fin = ctypes.c_int32()
    ms = (ctypes.c_double * 2)()
    s = 0 if stream is None else stream.cuda_stream
    _lib.check(batch.L.sg_autotune(batch.h, reps, tj, ctypes.byref(fin), ms,
                                   ctypes.c_void_p(s)), "sg_autotune")
    on = ctypes.c_int32()
    _lib.check(batch.L.sg_sweep(batch.h, ctypes.byref(on)), "sg_sweep")
    entry = {"tj": list(tj), "finish": fin.value, "stage_ms": ms[0],
             "solve_ms": ms[1], "sweep": on.value}
    _store(path, k, entry)
    return dict(entry, cached=False)
