"""Reading scarf's zarr count stores on the device.

scarf keeps each assay's raw counts as a dense zarr v2 array (cells x genes,
chunks of 1000 x 1000, ``<u4``) compressed with Blosc LZ4 and bit shuffle
(``create_zarr_dataset``, scarf/writers.py:58-89, :164-204). This module reads
the chunk files of such an array from a directory store, decodes them on the
GPU (``sg_blosc_decode``) a band of chunk rows at a time, and turns each band
into CSR rows on the device (``sg_chunks_to_csr``), so that counts go from disk
to ``make_graph`` without a CPU decompression pass. Missing chunk files hold
the fill value, as zarr defines.
"""
from __future__ import annotations

import json
import os
from typing import Tuple

import numpy as np
import torch

from . import kernels as K

_DTYPES = {"<u4": 4, "<i4": 4}


def array_meta(store: str, array: str) -> dict:
    with open(os.path.join(store, array, ".zarray")) as f:
        meta = json.load(f)
    comp = meta.get("compressor") or {}
    if meta.get("zarr_format") != 2 or meta.get("order", "C") != "C" or meta.get("filters"):
        raise NotImplementedError(f"{array}: only C-order zarr v2 arrays without filters are read on the device")
    if meta["dtype"] not in _DTYPES or len(meta["shape"]) != 2:
        raise NotImplementedError(f"{array}: only 2-D 32-bit integer count arrays are read on the device")
    if comp and (comp.get("id") != "blosc" or comp.get("cname") != "lz4"):
        raise NotImplementedError(f"{array}: only Blosc-LZ4 chunks are decoded on the device")
    return meta


def read_counts_csr(store: str, array: str = "RNA/counts", device="cuda"
                    ) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor, int]:
    """The count array ``array`` of the directory store ``store`` as device
    CSR ``(indptr int64, indices int32, data int32, n_genes)``."""
    meta = array_meta(store, array)
    n_rows, n_cols = meta["shape"]
    cr, cc = meta["chunks"]
    fill = int(meta.get("fill_value") or 0)
    if fill != 0:
        raise NotImplementedError(f"{array}: a non-zero fill value")
    dev = torch.device(device)
    nrc, ncc = -(-n_rows // cr), -(-n_cols // cc)
    chunk_bytes = cr * cc * 4
    band = torch.empty(ncc * cr * cc, dtype=torch.int32, device=dev)
    ptrs, inds, dats = [], [], []
    base = 0
    for ci in range(nrc):
        frames, starts = [], []
        band.zero_()
        for cj in range(ncc):
            p = os.path.join(store, array, f"{ci}.{cj}")
            if os.path.exists(p):
                with open(p, "rb") as f:
                    frames.append(f.read())
                starts.append(cj * chunk_bytes)
        if frames:
            K.blosc_decode(frames, band.view(torch.uint8), starts)
        rows = min(cr, n_rows - ci * cr)
        ip, ind, dat = K.chunks_to_csr(band, rows, cr, cc, n_cols, indptr_base=base)
        base += int(ind.numel())
        ptrs.append(ip[:-1] if ci < nrc - 1 else ip)
        inds.append(ind.clone())
        dats.append(dat.clone())
    return torch.cat(ptrs), torch.cat(inds), torch.cat(dats), n_cols


def read_strings(store: str, array: str, device="cuda") -> np.ndarray:
    """A 1-D fixed-width string array (cell or feature ids) of the store,
    its chunks decoded on the device."""
    with open(os.path.join(store, array, ".zarray")) as f:
        meta = json.load(f)
    (n,), (c,) = meta["shape"], meta["chunks"]
    dt = np.dtype(meta["dtype"])
    nch = -(-n // c)
    frames, starts = [], []
    for i in range(nch):
        p = os.path.join(store, array, str(i))
        if os.path.exists(p):
            with open(p, "rb") as f:
                frames.append(f.read())
            starts.append(i * c * dt.itemsize)
    out = torch.zeros(max(1, nch * c * dt.itemsize), dtype=torch.uint8, device=torch.device(device))
    if frames:
        K.blosc_decode(frames, out, starts)
    return np.frombuffer(out.cpu().numpy().tobytes(), dtype=dt)[:n].copy()
