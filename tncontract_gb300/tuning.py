"""Committed autotuning of the Jacobi variant of ``tnc_svd_rows``.

The drop-in's truncating SVD (``tensor_svd`` / ``truncated_svd`` of
tncontract/tensor.py:915, 1137-1152, and the engine's bond factorisations)
orthogonalises the rows of a QR factor with ``tnc_svd_rows``, whose
``block_rows`` selects the kernel variant: the Gram-form block update
(``ROWS_GRAM``) or the row-by-row rotation kernel with 4- or 8-row
half-blocks.  Which is fastest depends on the dtype, the row count and the
row length.  ``generate()`` times every candidate once per bucket on the GPU
at hand (CUDA events, after a warm-up call) and writes the winners to
``svd_rows_tuning.json`` beside this file; ``lookup()`` reads that committed
table (rows and length rounded up to the next bucket), and ``_ops.svd_rows``
falls back to timing at run time only for shapes outside it.

Regenerate on the target GPU with ``python -m tncontract_gb300.tuning``.
"""
from __future__ import annotations

import json
import os
import threading

TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "svd_rows_tuning.json")
ROWS = (16, 32, 64, 128, 256, 512, 1024)
LENGTHS = (64, 128, 256, 512, 1024)
DTYPES = ("float32", "complex64", "float64", "complex128")
# longest rows of the row kernels (longer ones take the accumulating SVD)
MAX_LEN = {"float32": 1024, "complex64": 1024, "float64": 512, "complex128": 512}

_cache = None
_lock = threading.Lock()


def _bucket(v, edges):
    for e in edges:
        if v <= e:
            return e
    return None


def key(dtype_name, rows, length):
    """The table key of a problem: its rows and row length rounded up to the
    next bucket (None when beyond the largest)."""
    r, n = _bucket(rows, ROWS), _bucket(length, LENGTHS)
    if r is None or n is None:
        return None
    return "%s:%d:%d" % (dtype_name, r, n)


def load(path=TABLE):
    global _cache
    with _lock:
        if _cache is None:
            try:
                with open(path) as f:
                    _cache = json.load(f).get("choices", {})
            except (OSError, ValueError):
                _cache = {}
        return _cache


def lookup(dtype_name, rows, length, table=None):
    """The committed block_rows choice for rows x length (rows <= length),
    or None."""
    k = key(dtype_name, rows, length)
    if k is None:
        return None
    t = load() if table is None else table
    v = t.get(k)
    return int(v) if v is not None else None


def generate(path=TABLE, seed=0):
    """Time every candidate on every bucket of this GPU and write the table."""
    import numpy as np
    import torch
    from . import _lib as L
    from . import _ops
    rng = np.random.default_rng(seed)
    choices, times = {}, {}
    npdt = {"float32": np.float32, "complex64": np.complex64, "float64": np.float64, "complex128": np.complex128}
    for name in DTYPES:
        for n in LENGTHS:
            if n > MAX_LEN[name]:
                continue
            for r in ROWS:
                if r > n:
                    continue
                a = rng.standard_normal((r, n))
                if name.startswith("complex"):
                    a = a + 1j * rng.standard_normal((r, n))
                M = torch.from_numpy(a.astype(npdt[name])).cuda()
                best, best_ms, row = None, None, {}
                for h in _ops.TUNE_CANDIDATES:
                    _ops.svd_rows(M, block_rows=h)  # warm-up (first launch of the variant)
                    torch.cuda.synchronize()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    _ops.svd_rows(M, block_rows=h)
                    e1.record()
                    torch.cuda.synchronize()
                    ms = e0.elapsed_time(e1)
                    row[str(h)] = round(ms, 4)
                    if best_ms is None or ms < best_ms:
                        best, best_ms = h, ms
                k = key(name, r, n)
                choices[k] = best
                times[k] = row
    out = {"device": torch.cuda.get_device_name(0), "candidates": list(_ops.TUNE_CANDIDATES),
           "gram": L.ROWS_GRAM, "choices": choices, "ms": times}
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    global _cache
    with _lock:
        _cache = None
    return out


if __name__ == "__main__":
    res = generate()
    print("%d buckets written to %s (%s)" % (len(res["choices"]), TABLE, res["device"]))
