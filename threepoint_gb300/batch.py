"""Checkpointed batch evaluation of <Map^3> over many cosmologies.

The reference writes its results only at the end of a run
(calculateApertureStatistics.cu:118-130), so an interrupted run restarts from
zero. Here a batch of cosmologies x aperture-radius triplets is evaluated in
chunks of cosmologies; every finished chunk is saved as
``chunk_<first>_<last>.npz`` (values, error estimates, evaluation counts, cap
status) and recorded in ``manifest.json`` together with a hash of the inputs.
Running the same batch again into the same directory skips the chunks already
there, so a killed run resumes where it stopped; a directory written for other
inputs is refused. Under a torch.distributed group each rank takes its
contiguous block of cosmologies (threepoint_gb300.shard.shard_range) and
writes its own chunks; rank 0 can assemble the result once all are present.
"""
from __future__ import annotations

import hashlib
import json
import os
from dataclasses import asdict, is_dataclass
from typing import Callable, Sequence

import numpy as np

MANIFEST = "manifest.json"


def inputs_hash(cosmologies: Sequence, thetas, extra: dict) -> str:
    h = hashlib.sha256()
    rows = [asdict(c) if is_dataclass(c) else dict(c) for c in cosmologies]
    h.update(json.dumps(rows, sort_keys=True).encode())
    h.update(np.ascontiguousarray(thetas, dtype=np.float64).tobytes())
    h.update(json.dumps(extra, sort_keys=True).encode())
    return h.hexdigest()


def _chunk_name(lo: int, hi: int) -> str:
    return f"chunk_{lo:06d}_{hi - 1:06d}.npz"


def _manifest_path(out_dir: str, rank: int) -> str:
    # each rank keeps its own manifest file; assemble() merges them
    return os.path.join(out_dir, MANIFEST if rank == 0 else f"manifest.rank{rank}.json")


def _load_manifest(out_dir: str, digest: str, n_cosmo: int, n_trip: int, chunk: int, rank: int) -> dict:
    for path in (os.path.join(out_dir, MANIFEST), _manifest_path(out_dir, rank)):
        if os.path.exists(path):
            with open(path) as f:
                other = json.load(f)
            if other.get("inputs") != digest or other.get("chunk") != chunk:
                raise ValueError(f"{out_dir} holds a batch of other inputs or chunking; use a new directory")
    path = _manifest_path(out_dir, rank)
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {"inputs": digest, "n_cosmo": n_cosmo, "n_triplets": n_trip, "chunk": chunk, "done": {}}


def _save_manifest(out_dir: str, m: dict, rank: int) -> None:
    path = _manifest_path(out_dir, rank)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(m, f, indent=1)
    os.replace(tmp, path)


def run(cosmologies: Sequence, thetas, out_dir: str,
        evaluate: Callable[[Sequence, np.ndarray], dict], chunk: int = 64, extra: dict | None = None,
        rank: int = 0, world: int = 1, progress: Callable[[int, int], None] | None = None) -> list:
    """Evaluate rank's block of ``cosmologies`` in chunks of ``chunk``.

    ``evaluate(cosmo_chunk, thetas)`` returns a dict of arrays with first axis
    len(cosmo_chunk) ("value" required; e.g. "err", "neval", "status").
    Returns the list of chunk files this rank wrote or found finished."""
    from .shard import shard_range

    th = np.ascontiguousarray(thetas, dtype=np.float64).reshape(-1, 3)
    os.makedirs(out_dir, exist_ok=True)
    digest = inputs_hash(cosmologies, th, extra or {})
    m = _load_manifest(out_dir, digest, len(cosmologies), len(th), chunk, rank)
    _save_manifest(out_dir, m, rank)
    lo_r, hi_r = shard_range(len(cosmologies), rank, world)
    files = []
    starts = list(range(lo_r - lo_r % chunk if lo_r % chunk else lo_r, hi_r, chunk))
    for s in starts:
        lo, hi = max(s, lo_r), min(s + chunk, hi_r)
        if lo >= hi:
            continue
        name = _chunk_name(lo, hi)
        path = os.path.join(out_dir, name)
        if m["done"].get(name) and os.path.exists(path):
            files.append(path)
            continue
        res = evaluate(list(cosmologies[lo:hi]), th)
        if "value" not in res:
            raise ValueError("evaluate() must return a 'value' array")
        arrays = {k: np.asarray(v) for k, v in res.items()}
        for k, v in arrays.items():
            if v.shape[0] != hi - lo:
                raise ValueError(f"evaluate() returned {k} with {v.shape[0]} rows for {hi - lo} cosmologies")
        tmp = path + ".tmp.npz"
        np.savez(tmp, lo=lo, hi=hi, **arrays)
        os.replace(tmp, path)
        m["done"][name] = [lo, hi]
        _save_manifest(out_dir, m, rank)
        files.append(path)
        if progress:
            progress(hi - lo_r, hi_r - lo_r)
    return files


def assemble(out_dir: str, key: str = "value") -> np.ndarray:
    """The [n_cosmo, n_triplets] array of ``key`` from all chunk files; raises
    if a cosmology is missing."""
    with open(os.path.join(out_dir, MANIFEST)) as f:
        m = json.load(f)
    done = dict(m["done"])
    for fn in os.listdir(out_dir):
        if fn.startswith("manifest.rank") and fn.endswith(".json"):
            with open(os.path.join(out_dir, fn)) as f:
                other = json.load(f)
            if other.get("inputs") != m["inputs"]:
                raise ValueError(f"{fn} belongs to another batch")
            done.update(other["done"])
    out = None
    seen = np.zeros(m["n_cosmo"], dtype=bool)
    for name, (lo, hi) in done.items():
        with np.load(os.path.join(out_dir, name)) as z:
            v = z[key]
        if out is None:
            out = np.zeros((m["n_cosmo"],) + v.shape[1:], dtype=v.dtype)
        out[lo:hi] = v
        seen[lo:hi] = True
    if out is None or not seen.all():
        raise RuntimeError(f"{out_dir}: {int((~seen).sum())} cosmologies not evaluated yet")
    return out


def context_evaluator(ctx, nz, precision: int = 1, **kw) -> Callable:
    """evaluate() for run(): one GPU context, all triplets of a chunk in one
    tp_map3_batch call (values, error estimates, evaluation counts, status)."""

    def evaluate(cosmos, th):
        ctx.set_cosmologies(cosmos, nz)
        v, info = ctx.map3_batch(th, precision=precision, return_info=True, check=False, **kw)
        return {"value": v, "err": info["err"], "neval": info["neval"], "status": info["status"]}

    return evaluate
