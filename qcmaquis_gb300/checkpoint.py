"""MPS checkpoints: save, load and resume.

Follows the reference's checkpoint layout (``mp_tensors/mps.hpp:312-365``,
``mp_tensors/mpstensor.hpp:544-565``, ``block_matrix/block_matrix.hpp:476-513``,
``sim/sim.hpp:165-215``): a directory with one file per site, ``mps<k>``, each
holding the site's physical, left and right indices and its left-paired block
matrix (row and column sector lists plus the dense blocks); every file is
written as ``<name>.new`` first and renamed once all sites are written, so an
interrupted save leaves the previous checkpoint readable; the number of sites
is found by probing the files; ``props`` holds the parameters, the version and
the sweep status.  The reference writes HDF5 through ALPS archives; HDF5 is not
a dependency here, so each site is one little-endian binary file:

    magic "QCMT", uint32 version
    3 indices (phys, left, right): int32 n, then n x (int32 N, int32 2S, int64 size)
    int32 nblocks, then nblocks x (int32 lc N, lc 2S, rc N, rc 2S, int64 rows, int64 cols)
    the blocks' elements, float64, column-major, in block order

and ``props.json`` is JSON.
"""
from __future__ import annotations

import json
import os
from typing import Dict, List, Optional, Tuple

import numpy as np

from .block_matrix import BlockMatrix
from .symmetry import Index

MAGIC = b"QCMT"
VERSION = 1


def _write_index(f, idx: Index):
    f.write(np.int32(len(idx.data)).tobytes())
    for (n, s2), size in idx.data:
        f.write(np.array([n, s2], dtype="<i4").tobytes())
        f.write(np.array([size], dtype="<i8").tobytes())


def _read_exact(f, n: int) -> bytes:
    b = f.read(n)
    if len(b) != n:
        raise ValueError("truncated checkpoint file")
    return b


def _read_index(f) -> Index:
    n = int(np.frombuffer(_read_exact(f, 4), dtype="<i4")[0])
    if n < 0:
        raise ValueError("corrupt checkpoint: negative sector count")
    out = []
    for _ in range(n):
        q = np.frombuffer(_read_exact(f, 8), dtype="<i4")
        s = int(np.frombuffer(_read_exact(f, 8), dtype="<i8")[0])
        out.append(((int(q[0]), int(q[1])), s))
    return Index.from_sorted(out)


def write_tensor(path: str, phys: Index, left: Index, right: Index, data: BlockMatrix):
    """One site: indices and the left-paired block matrix."""
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.uint32(VERSION).tobytes())
        for idx in (phys, left, right):
            _write_index(f, idx)
        f.write(np.int32(data.n_blocks()).tobytes())
        for (lc, rc), b in zip(data.keys, data.blocks):
            f.write(np.array([lc[0], lc[1], rc[0], rc[1]], dtype="<i4").tobytes())
            f.write(np.array(b.shape, dtype="<i8").tobytes())
        for b in data.blocks:
            f.write(np.asfortranarray(b, dtype="<f8").tobytes(order="F"))


def read_tensor(path: str):
    """(phys, left, right, BlockMatrix) of one site file."""
    with open(path, "rb") as f:
        if _read_exact(f, 4) != MAGIC:
            raise ValueError(f"{path}: not an MPS tensor checkpoint")
        ver = int(np.frombuffer(_read_exact(f, 4), dtype="<u4")[0])
        if ver != VERSION:
            raise ValueError(f"{path}: unsupported checkpoint version {ver}")
        phys, left, right = _read_index(f), _read_index(f), _read_index(f)
        nb = int(np.frombuffer(_read_exact(f, 4), dtype="<i4")[0])
        heads = []
        for _ in range(nb):
            q = np.frombuffer(_read_exact(f, 16), dtype="<i4")
            r, c = np.frombuffer(_read_exact(f, 16), dtype="<i8")
            if r < 0 or c < 0:
                raise ValueError("corrupt checkpoint: negative block shape")
            heads.append((((int(q[0]), int(q[1])), (int(q[2]), int(q[3]))), int(r), int(c)))
        bm = BlockMatrix()
        for (lc, rc), r, c in heads:
            a = np.frombuffer(_read_exact(f, 8 * r * c), dtype="<f8").reshape((r, c), order="F")
            bm.insert_block(np.array(a, dtype=np.float64), lc, rc)
        if f.read(1):
            raise ValueError(f"{path}: trailing bytes")
    return phys, left, right, bm


def _host(t):
    """(phys, left, right, left-paired BlockMatrix) of a device or host MPS tensor."""
    if hasattr(t, "to_block_matrix"):
        return t.phys_i, t.left_i, t.right_i, t.to_block_matrix()
    h = t.copy().make_left_paired()
    return h.phys_i, h.left_i, h.right_i, h.data


def save(dirname: str, mps, status: Optional[Dict] = None, parameters: Optional[Dict] = None):
    """``save`` + ``checkpoint_simulation``: every site file under its final name only after
    all of them are written, then the status."""
    os.makedirs(dirname, exist_ok=True)
    L = len(mps)
    for k, t in enumerate(mps):
        write_tensor(os.path.join(dirname, f"mps{k}.new"), *_host(t))
    for k in range(L):
        os.replace(os.path.join(dirname, f"mps{k}.new"), os.path.join(dirname, f"mps{k}"))
    # a longer earlier checkpoint in the same directory must not leave extra sites behind
    k = L
    while os.path.exists(os.path.join(dirname, f"mps{k}")):
        os.remove(os.path.join(dirname, f"mps{k}"))
        k += 1
    props = {"version": VERSION, "status": status or {}, "parameters": parameters or {}}
    tmp = os.path.join(dirname, "props.json.new")
    with open(tmp, "w") as f:
        json.dump(props, f)
    os.replace(tmp, os.path.join(dirname, "props.json"))


def load(dirname: str):
    """``load``: (list of (phys, left, right, BlockMatrix), status, parameters)."""
    L = 0
    while os.path.exists(os.path.join(dirname, f"mps{L}")):
        L += 1
    if L == 0:
        raise FileNotFoundError(f"no MPS checkpoint in {dirname}")
    sites = [read_tensor(os.path.join(dirname, f"mps{k}")) for k in range(L)]
    props = {}
    pp = os.path.join(dirname, "props.json")
    if os.path.exists(pp):
        with open(pp) as f:
            props = json.load(f)
    return sites, props.get("status", {}), props.get("parameters", {})


def to_device(sites, device="cuda"):
    """Device MPS tensors from loaded sites."""
    from . import native as N
    import torch
    from .engine import DeviceMPSTensor
    out = []
    for phys, left, right, bm in sites:
        lay = N.Layout.of(bm)
        out.append(DeviceMPSTensor(phys, left, right, lay, torch.from_numpy(lay.pack(bm)).to(device)))
    return out


__all__ = ["save", "load", "to_device", "write_tensor", "read_tensor"]
