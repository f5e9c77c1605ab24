"""Shard merge of library artifacts, streamed (scripts/merge_shards.py:48-137).

A production library is built as shards (one npz per array task) and merged
into one artifact of up to ~10 GB.  ``merge_shards`` keeps the reference's
contract: every shard must carry the same (delta, Delta, b) grid, schema,
build seed, grid and uncertainty metadata; entries are de-duplicated by the
append key (free water once; otherwise kio to 4 decimals, rho to 1, V to 6,
madi/library.py:231-240), first occurrence wins; the merged file carries the
first shard's build metadata and the same npz keys.

Unlike the reference, which loads every shard into LibraryEntry objects and
re-saves them, the merge here never holds more than one chunk of rows of one
array: per-entry arrays are copied member by member, in row chunks, from each
shard into one uncompressed npz written as a stream (the signal matrix is
memory-mapped when the shard stores it uncompressed, the layout the reference's
artifact reader maps, tests/physics_audit/_artifact.py:52-103).

    python -m custom_madi_gb300.shards shard*.npz -o merged.npz [--require-shards N]
"""

from __future__ import annotations

import argparse
import glob
import json
import os
import re
import struct
import sys
import zipfile
from typing import Iterable, List, Optional, Sequence

import numpy as np

# Arrays with one row per library entry (axis 0); every other member is
# metadata shared by all shards.
ENTRY_ARRAYS = ("kios", "rhos", "Vs", "vis", "vectors", "nominal_kios", "nominal_rhos", "nominal_Vs", "weights",
                "pps", "kio_analytic_eq5", "is_free_water", "entry_metadata_json", "signal_imag", "signal_variance",
                "ensemble_means_subset")


def npz_member(path: str, name: str, mmap: bool = True) -> np.ndarray:
    """Array ``name`` of an npz file; memory-mapped (read-only) when the member
    is stored uncompressed, read whole otherwise."""
    member = f"{name}.npy"
    with zipfile.ZipFile(path) as zf:
        info = zf.getinfo(member)
        stored = info.compress_type == zipfile.ZIP_STORED
        if not (mmap and stored):
            with zf.open(member) as fh:
                return np.lib.format.read_array(fh, allow_pickle=False)
    with open(path, "rb") as fh:
        fh.seek(info.header_offset)
        local = fh.read(30)
        if len(local) != 30 or local[:4] != b"PK\x03\x04":
            raise ValueError(f"{path}: bad local header for {member}")
        name_len, extra_len = struct.unpack("<HH", local[26:30])
        fh.seek(info.header_offset + 30 + name_len + extra_len)
        version = np.lib.format.read_magic(fh)
        if version == (1, 0):
            shape, fortran, dtype = np.lib.format.read_array_header_1_0(fh)
        elif version == (2, 0):
            shape, fortran, dtype = np.lib.format.read_array_header_2_0(fh)
        else:
            fh.seek(0)
            with zipfile.ZipFile(path) as zf, zf.open(member) as mh:
                return np.lib.format.read_array(mh, allow_pickle=False)
        offset = fh.tell()
    if dtype.hasobject:
        raise ValueError(f"{path}:{member} holds Python objects")
    if int(np.prod(shape)) == 0:
        return np.zeros(shape, dtype)
    return np.memmap(path, dtype=dtype, mode="r", offset=offset, shape=shape, order="F" if fortran else "C")


def _members(path: str) -> List[str]:
    with zipfile.ZipFile(path) as zf:
        return [n[:-4] for n in zf.namelist() if n.endswith(".npy")]


def _meta_signature(path: str) -> tuple:
    from .library import load_library_meta
    m = load_library_meta(path)
    bm = m.get("build_metadata") or {}
    return (json.dumps(m.get("delta_pairs")), json.dumps([float(b) for b in (m.get("b_values") or [])]),
            m.get("library_schema"), bm.get("build_seed"), json.dumps(bm.get("grid", {}), sort_keys=True),
            json.dumps(bm.get("uncertainty", {}), sort_keys=True))


def entry_keys(kios, rhos, Vs, free) -> list:
    """Append / de-duplication keys of the entries (madi/library.py:231-240)."""
    return [("free_water",) if bool(f) else (round(float(k), 4), round(float(r), 1), round(float(v), 6))
            for k, r, v, f in zip(kios, rhos, Vs, free)]


def expand_shards(patterns: Sequence[str]) -> List[str]:
    paths = []
    for pat in patterns:
        hit = sorted(glob.glob(pat))
        paths.extend(hit if hit else ([pat] if os.path.exists(pat) else []))
    return paths


def check_coverage(paths: Sequence[str], n_shards: int) -> None:
    """Every shard id 0..n-1 exactly once (ids from '.shard<k>' in the file names)."""
    found = []
    for p in paths:
        m = re.search(r"\.shard(\d+)(?:\.|$)", os.path.basename(p))
        if m is None:
            raise ValueError(f"cannot infer shard id from {p}")
        found.append(int(m.group(1)))
    if sorted(found) != list(range(n_shards)):
        raise ValueError(f"shard coverage mismatch; found={sorted(found)}, expected={list(range(n_shards))}")


class _StreamWriter:
    """An uncompressed npz written member by member; each array's header goes
    first, then its rows in any number of chunks."""

    def __init__(self, path: str):
        self.zf = zipfile.ZipFile(path, "w", compression=zipfile.ZIP_STORED, allowZip64=True)

    def begin(self, name: str, dtype: np.dtype, shape: tuple):
        self.fh = self.zf.open(f"{name}.npy", "w", force_zip64=True)
        header = {"descr": np.lib.format.dtype_to_descr(np.dtype(dtype)), "fortran_order": False,
                  "shape": tuple(int(x) for x in shape)}
        np.lib.format.write_array_header_2_0(self.fh, header)
        self.dtype = np.dtype(dtype)

    def rows(self, a: np.ndarray):
        self.fh.write(np.ascontiguousarray(a, dtype=self.dtype).tobytes())

    def end(self):
        self.fh.close()

    def whole(self, name: str, a: np.ndarray):
        a = np.asarray(a)
        self.begin(name, a.dtype, a.shape)
        self.rows(a)
        self.end()

    def close(self):
        self.zf.close()


def merge_shards(paths: Sequence[str], out: str, *, require_shards: Optional[int] = None,
                 chunk_rows: int = 4096, verbose: bool = True) -> dict:
    """Merge shard artifacts into ``out``; returns counts per shard."""
    paths = list(paths)
    if not paths:
        raise ValueError("no shard files")
    if require_shards is not None:
        check_coverage(paths, int(require_shards))
    sig0 = _meta_signature(paths[0])
    members0 = _members(paths[0])
    seen, keep, report = set(), [], []
    for p in paths:
        if _meta_signature(p) != sig0:
            raise ValueError(f"shard metadata/schema/uncertainty mismatch: {p}")
        if set(_members(p)) != set(members0):
            raise ValueError(f"shard {p} has a different array set than {paths[0]}")
        free = npz_member(p, "is_free_water", mmap=False) if "is_free_water" in members0 else None
        k, r, v = (npz_member(p, n, mmap=False) for n in ("kios", "rhos", "Vs"))
        if free is None:
            free = np.zeros(len(k), bool)
        mask = np.zeros(len(k), bool)
        for i, key in enumerate(entry_keys(k, r, v, free)):
            if key not in seen:
                seen.add(key)
                mask[i] = True
        keep.append(mask)
        report.append({"path": p, "entries": int(len(k)), "new": int(mask.sum())})
        if verbose:
            print(f"  {p}: +{int(mask.sum())} new  ({len(k)} in file)")
    n_total = int(sum(int(m.sum()) for m in keep))
    os.makedirs(os.path.dirname(os.path.abspath(out)) or ".", exist_ok=True)
    w = _StreamWriter(out)
    try:
        weights_all = []
        for name in members0:
            if name in ENTRY_ARRAYS:
                parts = [npz_member(p, name) for p in paths]
                dtype = np.result_type(*[a.dtype for a in parts])      # strings: the longest width
                tail = parts[0].shape[1:]
                if any(a.shape[1:] != tail for a in parts):
                    raise ValueError(f"shards disagree on the shape of {name}")
                w.begin(name, dtype, (n_total, *tail))
                for a, m in zip(parts, keep):
                    for s in range(0, len(m), chunk_rows):
                        mm = m[s:s + chunk_rows]
                        if mm.any():
                            rows = np.asarray(a[s:s + chunk_rows])[mm]
                            w.rows(rows)
                            if name == "weights":
                                weights_all.append(np.asarray(rows, float))
                w.end()
                del parts
            elif name == "has_weights":
                continue                                    # recomputed over the merged entries
            else:
                w.whole(name, npz_member(paths[0], name, mmap=False))
        if "has_weights" in members0:
            wv = np.concatenate(weights_all) if weights_all else np.zeros(0)
            w.whole("has_weights", np.array(bool(np.all(np.isfinite(wv)))))
    finally:
        w.close()
    if verbose:
        print(f"Merged library -> {out} ({n_total} entries)")
    return {"entries": n_total, "shards": report}


def main(argv: Optional[Iterable[str]] = None) -> int:
    ap = argparse.ArgumentParser(description="Merge per-shard MADI libraries into one npz (streamed).")
    ap.add_argument("shards", nargs="+", help="per-shard .npz files (globs allowed)")
    ap.add_argument("-o", "--out", required=True, help="merged library .npz")
    ap.add_argument("--require-shards", type=int, default=None,
                    help="require shard ids 0..N-1 exactly once before merging")
    ap.add_argument("--chunk-rows", type=int, default=4096)
    args = ap.parse_args(list(argv) if argv is not None else None)
    paths = expand_shards(args.shards)
    if not paths:
        print("ERROR: no shard files found")
        return 1
    try:
        merge_shards(paths, args.out, require_shards=args.require_shards, chunk_rows=args.chunk_rows)
    except ValueError as exc:
        print(f"ERROR: {exc}")
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
