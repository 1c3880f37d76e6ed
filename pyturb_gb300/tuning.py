"""Autotuning of launch schedules, cached per (device, workload, n, batch).

The knobs change how work is scheduled, never what is computed (results
agree to float32 rounding):

- the radix plan of the mixed-radix Stockham transform (sizes other than
  powers of two up to 4096, e.g. 384 = 3 x 2^7): which radices 8/4/2 the
  power-of-two part is split into, and in which order the stages run;
- the column pass of power-of-two grids: register-fed or TMA-fed;
- the number of concurrent branches of a captured frame loop, or of streams
  of a ragged ensemble.

Each candidate is timed with CUDA events on the current stream (warm-up, then
the median of a few repetitions) and the fastest is kept. Choices are cached
in a JSON file, ``$PYTURB_GB300_TUNE_CACHE`` (default
``~/.cache/pyturb_gb300/tune.json``), keyed by device name, workload and
sizes, so later processes reuse them without timing.
"""

from __future__ import annotations

import ctypes as C
import json
import os
import statistics
import tempfile
from pathlib import Path
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple

from . import _lib
from .backend import torch_module

__all__ = ["cache_path", "time_ms", "choose", "radix_plans", "grid_radices", "set_grid_radices",
           "tune_grid"]


def cache_path() -> Path:
    env = os.environ.get("PYTURB_GB300_TUNE_CACHE")
    return Path(env).expanduser() if env else Path.home() / ".cache" / "pyturb_gb300" / "tune.json"


def _load() -> Dict[str, Any]:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(key: str, value: Any) -> None:
    path = cache_path()
    data = _load()
    data[key] = value
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=str(path.parent), suffix=".tmp")
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # an unwritable cache only costs a re-tune


def device_key() -> str:
    torch = torch_module()
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"


def time_ms(fn: Callable[[], Any], warmup: int = 2, reps: int = 5) -> float:
    """Median device time of ``fn`` in ms (CUDA events on the current stream)."""
    torch = torch_module()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    return float(statistics.median(out))


def choose(key: str, candidates: Sequence[Any], apply: Callable[[Any], None],
           run: Callable[[], Any], warmup: int = 2, reps: int = 5) -> Any:
    """The cached or fastest candidate for ``key``; ``apply(c)`` installs c
    and ``run()`` is the timed work. The winner is left installed."""
    full = f"{device_key()}|{key}"
    cands = [c for c in candidates]
    cached = _load().get(full)
    if cached is not None:
        pick = tuple(cached) if isinstance(cached, list) else cached
        if pick in cands:
            apply(pick)
            return pick
    best, best_ms = None, float("inf")
    for c in cands:
        apply(c)
        ms = time_ms(run, warmup, reps)
        if ms < best_ms:
            best, best_ms = c, ms
    apply(best)
    _store(full, list(best) if isinstance(best, tuple) else best)
    return best


# ------------------------------------------------------------------ radix plans
def _factor(n: int) -> Tuple[int, List[int]]:
    """(power of two exponent, other prime factors ascending)."""
    a = 0
    while n % 2 == 0:
        n //= 2
        a += 1
    rest, p = [], 3
    while p * p <= n:
        while n % p == 0:
            rest.append(p)
            n //= p
        p += 2
    if n > 1:
        rest.append(n)
    return a, rest


def radix_plans(n: int, limit: int = 12) -> List[Tuple[int, ...]]:
    """Candidate stage plans for an n-point transform: the power-of-two part
    split into radices 8/4/2 in a few ways, odd factors as their own stages,
    in descending, ascending, odd-first and odd-last orders."""
    a, odd = _factor(int(n))
    splits = []
    for n8 in range(a // 3, -1, -1):
        rem = a - 3 * n8
        for n4 in range(rem // 2, -1, -1):
            n2 = rem - 2 * n4
            if n2 <= 1:
                splits.append([8] * n8 + [4] * n4 + [2] * n2)
    plans: List[Tuple[int, ...]] = []
    for two in splits[:3]:
        for order in (sorted(two, reverse=True) + odd, odd + sorted(two, reverse=True),
                      sorted(two) + odd, sorted(two + odd, reverse=True)):
            t = tuple(order)
            if t and t not in plans:
                plans.append(t)
    return plans[:limit] or [(int(n),)]


def grid_radices(grid) -> Tuple[int, ...]:
    ns = C.c_int(0)
    buf = (C.c_int * 24)()
    _lib.call("pt_grid_radices", grid.handle, C.byref(ns), buf)
    return tuple(buf[i] for i in range(ns.value))


def set_grid_radices(grid, plan: Sequence[int]) -> None:
    arr = (C.c_int * len(plan))(*[int(r) for r in plan])
    _lib.call("pt_grid_set_radices", grid.handle, len(plan), arr)


def tune_grid(grid, run: Callable[[], Any], batch: int, workload: str = "generate") -> Dict[str, Any]:
    """Tune one grid for ``run`` (the work it will repeat, on ``batch``
    screens): the radix plan of mixed-radix sizes, or the column-pass variant
    of power-of-two sizes that have both. Returns the choices."""
    n = grid.ns
    out: Dict[str, Any] = {}
    pow2 = n >= 8 and (n & (n - 1)) == 0 and n <= 4096
    # generate at n = 3 * 2^k (2^k in 64 .. 512) runs the Good-Thomas register
    # transforms, which have no radix plan to choose
    m3 = n // 3
    if workload in ("generate", "ragged") and n % 3 == 0 and 64 <= m3 <= 512 and (m3 & (m3 - 1)) == 0:
        return out
    if not pow2:
        default = grid_radices(grid)
        cands = radix_plans(n)
        if default not in cands:
            cands = [default] + cands
        out["radices"] = choose(f"{workload}|radices|n={n}|batch={batch}|P={grid.P}", cands,
                                lambda p: set_grid_radices(grid, p), run)
    elif n in (256, 512, 1024):
        out["cols_variant"] = choose(
            f"{workload}|cols|n={n}|batch={batch}|P={grid.P}", [0, 1],
            lambda v: _lib.call("pt_grid_set_cols_variant", grid.handle, int(v)), run)
    return out
