"""Writing scarf's zarr format on the device (f2, the writing half:
create_zarr_dataset, scarf/writers.py:58-89, :164-204). Every frame the
device encoder writes must follow the Blosc1 and LZ4 formats (header fields,
the LZ4 end-of-block rules) and decode, with the oracle's CPU decoder and
with the device decoder, to the bytes that went in; arrays and whole
DataStores written as zarr stores read back unchanged."""
import json
import os

import numpy as np
import pytest

from helpers import check_frame, small_counts, top_var_genes
from oracle import blosc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def K():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300 import kernels
    return kernels


def _cases(rng):
    out = []
    for ts in (1, 2, 4, 8, 12):
        for n in (0, 1, 5, 13, 97, 4096, 32768 // ts, 32768 // ts + 3, 70001):
            nb = n * ts
            out.append(("random", ts, rng.integers(0, 256, nb, dtype=np.uint8).tobytes()))
            out.append(("zeros", ts, bytes(nb)))
            out.append(("counts", ts, rng.poisson(0.3, nb).astype(np.uint8).tobytes()))
    idx = np.sort(rng.integers(0, 1_000_000, 50_000)).astype(np.int64)
    out.append(("sorted u8", 8, idx.tobytes()))
    out.append(("weights f8", 8, rng.random(30_000).astype(np.float64).tobytes()))
    out.append(("edges", 8, np.repeat(np.arange(20_000, dtype=np.int64), 21).tobytes()))
    return out


def test_frames_follow_the_format_and_round_trip(K):
    rng = np.random.default_rng(3)
    cases = _cases(rng)
    for shuffle in (2, 1, 0):
        for bs in (32768, 4096, 200):
            sub = [(name, ts, d) for name, ts, d in cases if bs % ts == 0]
            for ts in sorted({ts for _, ts, _ in sub}):
                datas = [d for _, t, d in sub if t == ts]
                buf = np.frombuffer(b"".join(datas) or b"\0", dtype=np.uint8)
                offs = np.concatenate([[0], np.cumsum([len(d) for d in datas])]).astype(np.int64)
                frames = K.blosc_encode(torch.from_numpy(buf.copy()).cuda(), offs, ts, shuffle, bs)
                assert len(frames) == len(datas)
                for fr, d in zip(frames, datas):
                    hdr = check_frame(fr)
                    assert hdr["nbytes"] == len(d) and hdr["typesize"] == ts
                    want_flag = 0 if ts == 1 else {2: 0x04, 1: 0x01, 0: 0}[shuffle]
                    assert hdr["flags"] & 0x05 == want_flag and hdr["flags"] & 0x10
                    assert blosc.decompress(fr) == d
                # and the device decoder reads them back
                nz = [(fr, d) for fr, d in zip(frames, datas) if d]
                starts = np.concatenate([[0], np.cumsum([len(d) for _, d in nz])[:-1]]).astype(np.int64)
                out = torch.zeros(max(1, sum(len(d) for _, d in nz)), dtype=torch.uint8, device="cuda")
                K.blosc_decode([fr for fr, _ in nz], out, starts)
                torch.cuda.synchronize()
                assert out.cpu().numpy().tobytes()[:sum(len(d) for _, d in nz)] == b"".join(d for _, d in nz)


def test_compressible_data_compresses(K):
    counts = np.random.default_rng(1).poisson(0.2, (1000, 1000)).astype(np.uint32)
    for arr, most in ((np.zeros(1 << 20, np.uint8), 0.01), (counts, 0.35)):
        b = torch.from_numpy(arr.reshape(-1).view(np.uint8).copy()).cuda()
        fr = K.blosc_encode(b, np.array([0, b.numel()]), arr.dtype.itemsize, 2)[0]
        assert len(fr) < most * b.numel(), (arr.dtype, len(fr))
        assert blosc.decompress(fr) == arr.tobytes()


def test_bad_arguments_are_refused(K):
    from scarf_gb300 import _lib as L
    b = torch.zeros(64, dtype=torch.uint8, device="cuda")
    offs = np.array([0, 64], dtype=np.int64)
    fo = np.zeros(2, np.int64)
    big, small = np.zeros(200, np.uint8), np.zeros(10, np.uint8)
    lib, h = L.load(), K.handle(0).ptr
    for bs, out in ((60, big), (64, small)):    # a block size not a multiple of 8; too small a capacity
        with pytest.raises(ValueError):
            L.check(lib.sg_blosc_encode(h, b.data_ptr(), offs.ctypes.data, 1, 8, 2, bs, out.ctypes.data, out.size,
                                        fo.ctypes.data, None))


def test_arrays_round_trip_through_a_store(K, tmp_path):
    from scarf_gb300.zarr_io import read_array, write_array
    rng = np.random.default_rng(7)
    arrays = {
        "a/f8": (rng.random((2503, 21)), (1000, 21)),
        "a/u8": (rng.integers(0, 10**6, (777, 2)).astype(np.uint64), (100, 2)),
        "b/i4": (rng.integers(-5, 5, (33, 1001)).astype(np.int32), (10, 300)),
        "b/bool": (rng.random(5000) < 0.3, (1000,)),
        "c/ids": (np.array([f"cell_{i}-1" for i in range(1234)]), (500,)),
    }
    for name, (a, ch) in arrays.items():
        write_array(str(tmp_path), name, a, chunks=ch, shuffle=1 if a.dtype.kind == "U" else 2,
                    attrs={"note": name})
        got = read_array(str(tmp_path), name)
        assert got.dtype == a.dtype and np.array_equal(got, a), name
        meta = json.loads((tmp_path / name / ".zarray").read_text())
        assert meta["compressor"]["cname"] == "lz4" and meta["chunks"] == list(ch)
        # every chunk file is a valid frame the oracle decodes
        for f in os.listdir(tmp_path / name):
            if not f.startswith("."):
                check_frame((tmp_path / name / f).read_bytes())
    # a device tensor, padded edge chunks included
    t = torch.arange(10_007 * 3, dtype=torch.float32, device="cuda").reshape(10_007, 3)
    write_array(str(tmp_path), "dev/t", t, chunks=(4096, 3))
    assert np.array_equal(read_array(str(tmp_path), "dev/t"), t.cpu().numpy())


def test_datastore_to_zarr_round_trip(K, tmp_path):
    from scarf_gb300.datastore import DataStore
    from scarf_gb300.zarr_io import read_array
    indptr, indices, data, G, _ = small_counts(n_cells=1500, n_genes=2500, seed=5)
    feat = top_var_genes(indptr, indices, data, G, 200)
    ids = np.array([f"g{i}" for i in range(G)])
    cells = np.array([f"c{i}-1" for i in range(len(indptr) - 1)])
    d = DataStore(indptr, indices, data, G, gene_ids=ids, cell_ids=cells, precision="precision")
    mask = np.zeros(G, dtype=bool)
    mask[feat] = True
    d.RNA.feats.insert("I__hvgs", mask)
    d.make_graph(feat_key="hvgs", dims=12, k=9, batch_size=500)
    store = str(tmp_path / "ds.zarr")
    d.to_zarr(store)
    # the counts in scarf's layout, as the reference's own store has them
    meta = json.loads(open(os.path.join(store, "RNA", "counts", ".zarray")).read())
    assert meta["dtype"] == "<u4" and meta["chunks"] == [1000, 1000] and meta["compressor"]["shuffle"] == 2
    back = DataStore.from_zarr(store)
    assert np.array_equal(back.RNA.indptr, d.RNA.indptr)
    assert np.array_equal(back.RNA.indices, d.RNA.indices) and np.array_equal(back.RNA.data, d.RNA.data)
    assert np.array_equal(back.cells.fetch_all("ids"), cells)
    assert np.array_equal(back.RNA.feats.fetch_all("ids"), ids)
    assert np.array_equal(read_array(store, "RNA/featureData/I__hvgs"), mask)
    # the graph datasets
    found = 0
    for root, dirs, files in os.walk(store):
        rel = os.path.relpath(root, store)
        if ".zarray" in files and rel.split(os.sep)[-1] in ("indices", "distances", "edges", "weights"):
            want = np.asarray(d.zw[rel.replace(os.sep, "/")])
            assert np.array_equal(read_array(store, rel), want), rel
            found += 1
    assert found == 4, found
    attrs = json.loads(open(os.path.join(store, "RNA", ".zattrs")).read())
    assert attrs["size_factor"] == 1000
