"""Reading and writing scarf's zarr stores on the device.

scarf keeps each assay's raw counts as a dense zarr v2 array (cells x genes,
chunks of 1000 x 1000, ``<u4``) compressed with Blosc LZ4 and bit shuffle
(``create_zarr_dataset``, scarf/writers.py:58-89, :164-204). This module reads
the chunk files of such an array from a directory store, decodes them on the
GPU (``sg_blosc_decode``) a band of chunk rows at a time, and turns each band
into CSR rows on the device (``sg_chunks_to_csr``), so that counts go from disk
to ``make_graph`` without a CPU decompression pass. Missing chunk files hold
the fill value, as zarr defines.

Writing goes the other way: ``write_array`` / ``write_group`` lay an array
(or a whole in-memory store group) out in zarr v2 chunks and encode every
chunk on the GPU (``sg_blosc_encode``) as the Blosc-LZ4 bit-shuffle frames
scarf's ``create_zarr_dataset`` writes, so that scarf, zarr or this module
read the result back. ``read_array`` reads any such array.
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


# scarf's compressor settings (scarf/writers.py:79-89)
BLOSC = {"id": "blosc", "cname": "lz4", "clevel": 5, "shuffle": 2, "blocksize": 0}
WRITE_BATCH_BYTES = 1 << 28   # chunks encoded per device batch


def _chunk_indices(shape, chunks):
    grid = [max(1, -(-s // c)) for s, c in zip(shape, chunks)]
    return list(np.ndindex(*grid)) if shape else [()]


def _fill_json(v, dt):
    if dt.kind == "f" and v is not None and np.isnan(v):
        return "NaN"
    if dt.kind in "US":
        return ""
    return None if v is None else v.item() if hasattr(v, "item") else v


def write_array(store: str, name: str, data, chunks=None, attrs=None, shuffle: int = 2,
                blocksize: int = 32768, fill_value=0, device="cuda") -> None:
    """``data`` (numpy array or device tensor) as the zarr v2 array ``name``
    of the directory store ``store``: C order, chunks of ``chunks`` (default
    the whole array), every chunk a Blosc-LZ4 frame encoded on the device
    (bit shuffle unless ``shuffle`` says otherwise). Edge chunks are padded
    with ``fill_value``, as zarr stores them."""
    dev = torch.device(device)
    if isinstance(data, torch.Tensor):
        a_np = None
        t = data.detach().to(dev).contiguous()
        dt = np.dtype(str(t.dtype).replace("torch.", "").replace("bool", "bool_")) if t.dtype != torch.bool \
            else np.dtype(bool)
        shape = tuple(t.shape)
    else:
        a_np = np.ascontiguousarray(data)
        dt = a_np.dtype
        shape = a_np.shape
    chunks = tuple(int(c) for c in (chunks or shape or (1,)))
    if len(chunks) > len(shape):
        raise ValueError("more chunk lengths than dimensions")
    chunks = chunks + tuple(shape[len(chunks):])   # as zarr: trailing dimensions whole
    chunks = tuple(max(1, min(c, s)) if s else max(1, c) for c, s in zip(chunks, shape))
    path = os.path.join(store, name)
    os.makedirs(path, exist_ok=True)
    meta = {"zarr_format": 2, "shape": list(shape), "chunks": list(chunks), "dtype": dt.str,
            "compressor": dict(BLOSC, shuffle=int(shuffle)), "fill_value": _fill_json(fill_value, dt),
            "order": "C", "filters": None}
    with open(os.path.join(path, ".zarray"), "w") as f:
        json.dump(meta, f)
    if attrs:
        with open(os.path.join(path, ".zattrs"), "w") as f:
            json.dump(attrs, f, default=_jsonable)
    if 0 in shape:
        return
    ts = dt.itemsize if dt.itemsize <= 255 else 1
    cbytes = int(np.prod(chunks)) * dt.itemsize
    idxs = _chunk_indices(shape, chunks)
    per_batch = max(1, WRITE_BATCH_BYTES // max(1, cbytes))
    for b0 in range(0, len(idxs), per_batch):
        batch = idxs[b0:b0 + per_batch]
        if a_np is not None:     # chunks assembled on the host, one copy to the device
            host = np.empty((len(batch),) + chunks, dtype=dt)
            host[...] = np.array(fill_value if fill_value is not None else 0).astype(dt) if dt.kind not in "US" else ""
            for i, ix in enumerate(batch):
                sl = tuple(slice(j * c, min((j + 1) * c, s)) for j, c, s in zip(ix, chunks, shape))
                host[(i,) + tuple(slice(0, x.stop - x.start) for x in sl)] = a_np[sl]
            buf = torch.from_numpy(host.reshape(-1).view(np.uint8)).to(dev)
        else:                    # chunks assembled on the device
            dbuf = torch.full((len(batch),) + chunks, fill_value if fill_value is not None else 0, dtype=t.dtype,
                              device=dev)
            for i, ix in enumerate(batch):
                sl = tuple(slice(j * c, min((j + 1) * c, s)) for j, c, s in zip(ix, chunks, shape))
                dbuf[(i,) + tuple(slice(0, x.stop - x.start) for x in sl)] = t[sl]
            buf = dbuf.reshape(-1).view(torch.uint8)
        offs = np.arange(len(batch) + 1, dtype=np.int64) * cbytes
        frames = K.blosc_encode(buf, offs, ts, shuffle if dt.itemsize > 1 else 0, blocksize)
        for ix, fr in zip(batch, frames):
            with open(os.path.join(path, ".".join(str(j) for j in ix) or "0"), "wb") as f:
                f.write(fr)


def _jsonable(o):
    if isinstance(o, np.integer):
        return int(o)
    if isinstance(o, np.floating):
        return float(o)
    if isinstance(o, np.ndarray):
        return o.tolist()
    if isinstance(o, (np.bool_,)):
        return bool(o)
    raise TypeError(type(o))


def write_group(store: str, group, path: str = "", device="cuda") -> None:
    """An in-memory store group (``scarf_gb300.store.Group``: attributes,
    sub-groups and arrays) as a zarr v2 directory store, every array chunk
    encoded on the device."""
    from .store import Array, Group
    d = os.path.join(store, path)
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, ".zgroup"), "w") as f:
        json.dump({"zarr_format": 2}, f)
    if group.attrs:
        with open(os.path.join(d, ".zattrs"), "w") as f:
            json.dump(group.attrs, f, default=_jsonable)
    for k in group.keys():
        v = group[k]
        sub = f"{path}/{k}" if path else k
        if isinstance(v, Group):
            write_group(store, v, sub, device)
        elif isinstance(v, Array):
            write_array(store, sub, np.asarray(v), chunks=v.chunks, attrs=v.attrs, device=device)


def read_array(store: str, name: str, device="cuda") -> np.ndarray:
    """Any zarr v2 array of the store with Blosc-LZ4 (or no) compression,
    its chunks decoded on the device."""
    with open(os.path.join(store, name, ".zarray")) as f:
        meta = json.load(f)
    comp = meta.get("compressor")
    if meta.get("order", "C") != "C" or meta.get("filters"):
        raise NotImplementedError(f"{name}: only C-order arrays without filters")
    if comp and (comp.get("id") != "blosc" or comp.get("cname") != "lz4"):
        raise NotImplementedError(f"{name}: only Blosc-LZ4 chunks are decoded on the device")
    dt = np.dtype(meta["dtype"])
    shape, chunks = tuple(meta["shape"]), tuple(meta["chunks"])
    fill = meta.get("fill_value")
    out = np.zeros(shape, dtype=dt)
    if fill not in (None, 0, "") and dt.kind not in "US":
        out[...] = np.nan if fill == "NaN" else fill
    if 0 in shape:
        return out
    cbytes = int(np.prod(chunks)) * dt.itemsize
    idxs = _chunk_indices(shape, chunks)
    frames, present = [], []
    for ix in idxs:
        p = os.path.join(store, name, ".".join(str(j) for j in ix) or "0")
        if os.path.exists(p):
            with open(p, "rb") as f:
                frames.append(f.read())
            present.append(ix)
    if not frames:
        return out
    if comp:
        buf = torch.zeros(len(frames) * cbytes, dtype=torch.uint8, device=torch.device(device))
        K.blosc_decode(frames, buf, np.arange(len(frames), dtype=np.int64) * cbytes)
        raw = buf.cpu().numpy()
    else:
        raw = np.frombuffer(b"".join(frames), dtype=np.uint8)
    for i, ix in enumerate(present):
        ch = raw[i * cbytes:(i + 1) * cbytes].view(dt).reshape(chunks)
        sl = tuple(slice(j * c, min((j + 1) * c, s)) for j, c, s in zip(ix, chunks, shape))
        out[sl] = ch[tuple(slice(0, x.stop - x.start) for x in sl)]
    return out


def write_counts(store: str, name: str, indptr, indices, data, n_cols: int, chunks=(1000, 1000),
                 device="cuda") -> None:
    """CSR counts (host or device arrays) as scarf's dense ``<u4`` count array
    (scarf/writers.py:164-204): each band of chunk rows is made dense on the
    device and its chunks are encoded there."""
    dev = torch.device(device)
    ip = torch.as_tensor(np.asarray(indptr, dtype=np.int64) if not isinstance(indptr, torch.Tensor) else indptr)
    ind = torch.as_tensor(indices if isinstance(indices, torch.Tensor) else np.asarray(indices, dtype=np.int32))
    dat = torch.as_tensor(data if isinstance(data, torch.Tensor) else np.asarray(data, dtype=np.int32))
    n_rows = ip.numel() - 1
    cr, cc = int(chunks[0]), int(chunks[1])
    path = os.path.join(store, name)
    os.makedirs(path, exist_ok=True)
    meta = {"zarr_format": 2, "shape": [n_rows, int(n_cols)], "chunks": [cr, cc], "dtype": "<u4",
            "compressor": dict(BLOSC), "fill_value": 0, "order": "C", "filters": None}
    with open(os.path.join(path, ".zarray"), "w") as f:
        json.dump(meta, f)
    ncc = max(1, -(-int(n_cols) // cc))
    ipn = ip.cpu().numpy()
    for ci in range(max(1, -(-n_rows // cr))):
        r0, r1 = ci * cr, min(n_rows, (ci + 1) * cr)
        if r0 >= r1:
            break
        a, b = int(ipn[r0]), int(ipn[r1])
        rows = torch.repeat_interleave(torch.arange(r1 - r0, device=dev),
                                       torch.as_tensor(np.diff(ipn[r0:r1 + 1]), device=dev))
        band = torch.zeros((cr, ncc * cc), dtype=torch.int32, device=dev)
        if b > a:
            band.view(-1).index_put_((rows * (ncc * cc) + ind[a:b].to(dev).long(),), dat[a:b].to(dev).int(),
                                     accumulate=True)
        # chunk cj of the band: rows x columns [cj*cc, (cj+1)*cc), contiguous
        chunks_dev = band.view(cr, ncc, cc).permute(1, 0, 2).contiguous()
        offs = np.arange(ncc + 1, dtype=np.int64) * (cr * cc * 4)
        frames = K.blosc_encode(chunks_dev.view(-1).view(torch.uint8), offs, 4, 2)
        for cj, fr in enumerate(frames):
            with open(os.path.join(path, f"{ci}.{cj}"), "wb") as f:
                f.write(fr)


def write_table(store: str, name: str, table, device="cuda") -> None:
    """A column table (cell or feature metadata) as 1-D arrays
    ``{name}/{column}``; strings are written as fixed-width unicode with byte
    shuffle, as scarf stores its id columns."""
    os.makedirs(os.path.join(store, name), exist_ok=True)
    with open(os.path.join(store, name, ".zgroup"), "w") as f:
        json.dump({"zarr_format": 2}, f)
    for col in table.columns:
        v = np.asarray(table.fetch_all(col))
        if v.dtype == object:
            v = v.astype(str)
        write_array(store, f"{name}/{col}", v, chunks=(min(len(v), 100_000) or 1,),
                    shuffle=1 if v.dtype.kind in "US" else 2, device=device)
