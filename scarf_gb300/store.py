"""Hierarchical array store with the subset of the zarr group API that scarf's
graph path uses (``create_group``, ``create_dataset``, ``attrs``, path
indexing, ``in``, ``del``).

When zarr is importable, ``open_store(path)`` returns a real zarr group and
every writer here goes through it (Blosc-LZ4 bit-shuffle, as
``create_zarr_dataset`` does in scarf/writers.py:58-89). Otherwise an in-memory
``Group`` of numpy arrays is used, which can be saved to and loaded from a
directory of ``.npy`` files plus JSON attributes (checkpoint/resume of the
cached steps).
"""
from __future__ import annotations

import json
import os
from typing import Any, Dict, Optional, Tuple

import numpy as np


class Array:
    """A numpy-backed dataset with zarr-like slicing and attributes."""

    def __init__(self, shape, dtype, chunks=None):
        self._a = np.zeros(shape, dtype=np.dtype(dtype))
        self.chunks = tuple(chunks) if chunks is not None else tuple(shape)
        self.attrs: Dict[str, Any] = {}

    @property
    def shape(self) -> Tuple[int, ...]:
        return self._a.shape

    @property
    def dtype(self):
        return self._a.dtype

    def __getitem__(self, item):
        return self._a[item]

    def __setitem__(self, item, value):
        self._a[item] = value

    def __array__(self, dtype=None):
        return self._a if dtype is None else self._a.astype(dtype)

    def __len__(self):
        return self._a.shape[0]


class Group:
    def __init__(self, name: str = "/"):
        self.name = name
        self.attrs: Dict[str, Any] = {}
        self._children: Dict[str, Any] = {}

    # -- navigation -----------------------------------------------------------
    def _walk(self, path: str, create: bool = False):
        node = self
        parts = [p for p in path.strip("/").split("/") if p]
        for i, p in enumerate(parts):
            if p not in node._children:
                if not create:
                    raise KeyError(path)
                node._children[p] = Group(f"{node.name.rstrip('/')}/{p}")
            node = node._children[p]
            if isinstance(node, Array) and i != len(parts) - 1:
                raise KeyError(path)
        return node

    def __getitem__(self, path: str):
        return self._walk(path)

    def __contains__(self, path: str) -> bool:
        try:
            self._walk(path)
            return True
        except KeyError:
            return False

    def __delitem__(self, path: str):
        parts = [p for p in path.strip("/").split("/") if p]
        parent = self._walk("/".join(parts[:-1])) if len(parts) > 1 else self
        del parent._children[parts[-1]]

    def keys(self):
        return list(self._children)

    def __iter__(self):
        return iter(self._children)

    # -- creation -------------------------------------------------------------
    def create_group(self, path: str, overwrite: bool = False) -> "Group":
        if overwrite and path in self:
            del self[path]
        return self._walk(path, create=True)

    def require_group(self, path: str) -> "Group":
        return self._walk(path, create=True)

    def create_dataset(self, name: str, shape=None, dtype="f8", chunks=None, overwrite: bool = True,
                       compressor=None, **_kw) -> Array:
        parts = [p for p in name.strip("/").split("/") if p]
        parent = self._walk("/".join(parts[:-1]), create=True) if len(parts) > 1 else self
        if parts[-1] in parent._children and not overwrite:
            raise KeyError(f"{name} exists")
        arr = Array(shape, dtype, chunks)
        parent._children[parts[-1]] = arr
        return arr

    # -- persistence ----------------------------------------------------------
    def save(self, directory: str) -> None:
        os.makedirs(directory, exist_ok=True)
        with open(os.path.join(directory, ".attrs.json"), "w") as f:
            json.dump(self.attrs, f, default=_jsonable)
        for k, v in self._children.items():
            p = os.path.join(directory, k)
            if isinstance(v, Group):
                v.save(p)
            else:
                np.save(p + ".npy", v._a)
                with open(p + ".attrs.json", "w") as f:
                    json.dump({"chunks": list(v.chunks), "attrs": v.attrs}, f, default=_jsonable)


def _jsonable(o):
    if isinstance(o, (np.integer,)):
        return int(o)
    if isinstance(o, (np.floating,)):
        return float(o)
    if isinstance(o, np.ndarray):
        return o.tolist()
    raise TypeError(type(o))


def load_group(directory: str, name: str = "/") -> Group:
    g = Group(name)
    ap = os.path.join(directory, ".attrs.json")
    if os.path.exists(ap):
        with open(ap) as f:
            g.attrs = json.load(f)
    for entry in sorted(os.listdir(directory)):
        p = os.path.join(directory, entry)
        if os.path.isdir(p):
            g._children[entry] = load_group(p, f"{name.rstrip('/')}/{entry}")
        elif entry.endswith(".npy"):
            key = entry[:-4]
            a = np.load(p)
            arr = Array(a.shape, a.dtype)
            arr._a = a
            mp = os.path.join(directory, key + ".attrs.json")
            if os.path.exists(mp):
                with open(mp) as f:
                    meta = json.load(f)
                arr.chunks = tuple(meta.get("chunks", a.shape))
                arr.attrs = meta.get("attrs", {})
            g._children[key] = arr
    return g


def open_store(path: Optional[str] = None, mode: str = "a"):
    """A zarr group at ``path`` when zarr is installed, else an in-memory
    ``Group`` (loaded from ``path`` when it is a saved directory)."""
    if path is not None:
        try:
            import zarr  # noqa: F401
            return zarr.open_group(path, mode=mode)
        except ImportError:
            if os.path.isdir(path):
                return load_group(path)
    return Group()


def create_zarr_dataset(g, name: str, chunks: tuple, dtype: Any, shape: Tuple, overwrite: bool = True):
    """scarf/writers.py:58-89: a dataset of ``shape``/``dtype`` chunked along
    rows; Blosc-LZ4 bit-shuffle when the store is a zarr group."""
    if isinstance(dtype, tuple):
        dtype = dtype[0]
    if isinstance(g, Group):
        return g.create_dataset(name, shape=shape, dtype=dtype, chunks=chunks, overwrite=overwrite)
    try:
        from numcodecs import Blosc
        comp = Blosc(cname="lz4", clevel=5, shuffle=Blosc.BITSHUFFLE)
    except ImportError:
        comp = None
    return g.create_dataset(name, chunks=chunks, dtype=dtype, shape=shape, compressor=comp, overwrite=overwrite)
