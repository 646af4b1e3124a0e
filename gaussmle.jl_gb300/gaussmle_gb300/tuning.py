"""Autotuner front end: run gmle_autotune on a device batch and keep the
chosen launch shapes in a JSON cache keyed by GPU name, so later processes
start with them (gmle_set_tuning)."""
from __future__ import annotations

import ctypes as C
import json
import os
from pathlib import Path

from . import _lib

CACHE = Path(os.environ.get("GAUSSMLE_GB300_TUNING",
                            Path.home() / ".cache" / "gaussmle_gb300" / "tuning.json"))


def _gpu_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return f"cuda:{device}"


def _key(model: int, box: int, camera: int) -> str:
    return f"{model}/{box}/{int(camera != 0)}"


def load_cache(ctx: _lib.Context) -> int:
    """Apply cached shapes for this GPU to ctx; returns how many were applied."""
    if not CACHE.exists():
        return 0
    try:
        table = json.loads(CACHE.read_text()).get(_gpu_name(ctx.device), {})
    except (OSError, ValueError, AttributeError):
        return 0
    if not isinstance(table, dict):
        return 0
    k = 0
    for key, shape in table.items():
        try:
            m, b, cam = (int(v) for v in key.split("/"))
            tpr, rpb = (int(v) for v in shape)
        except (TypeError, ValueError):
            continue  # a malformed entry: keep the built-in default for that kind
        # the library validates the shape and rejects one it cannot launch
        if ctx.lib.gmle_set_tuning(ctx.handle, m, b, cam, tpr, rpb) == 0:
            k += 1
    return k


def autotune(ctx: _lib.Context, desc: _lib.FitDesc, data, xc, yc, params, crlb, llr,
             flags=None, save: bool = True) -> tuple[int, int, float]:
    """Time all launch shapes on the given CUDA tensors; keep and cache the best."""
    t, r, ms = C.c_int32(), C.c_int32(), C.c_float()
    p = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
    ctx.check(ctx.lib.gmle_autotune(ctx.handle, C.byref(desc), p(data), p(xc), p(yc),
                                    params.shape[0], p(params), p(crlb), p(llr), p(flags),
                                    C.byref(t), C.byref(r), C.byref(ms)))
    if save:
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            allt = json.loads(CACHE.read_text()) if CACHE.exists() else {}
            allt.setdefault(_gpu_name(ctx.device), {})[
                _key(desc.model, desc.box, desc.camera)] = [t.value, r.value]
            CACHE.write_text(json.dumps(allt, indent=1))
        except OSError:
            pass
    return t.value, r.value, ms.value
