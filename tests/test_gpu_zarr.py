"""Device-side reading of scarf's zarr count stores (Blosc1 / LZ4 / shuffles,
scarf/writers.py:58-89, :164-204): the GPU decoder bit for bit against the
oracle on the reference's own chunks and on frames of every layout, malformed
streams refused without a fault, and dense chunks to CSR on the device."""
import json
import os
import struct

import numpy as np
import pytest
import scipy.sparse as sp

from helpers import blosc_frame
from oracle import blosc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def z(golden_dir):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return np.load(os.path.join(golden_dir, "zarr_chunks.npz"))


def _decode(frames):
    from scarf_gb300 import kernels as K
    sizes = [blosc.parse_header(f)["nbytes"] for f in frames]
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    out = torch.zeros(max(1, int(sum(sizes))), dtype=torch.uint8, device="cuda")
    K.blosc_decode(frames, out, starts)
    torch.cuda.synchronize()
    host = out.cpu().numpy().tobytes()
    return [host[s:s + n] for s, n in zip(starts, sizes)]


def test_reference_chunks_decode_bit_exact(z):
    keys = ["rna_0_0", f"rna_0_{int(z['rna_last_chunk'])}", "adt_0_0", "cell_ids_0"]
    frames = [z[k].tobytes() for k in keys]
    for got, fr in zip(_decode(frames), frames):
        assert got == blosc.decompress(fr)


def test_frames_of_every_layout_decode_bit_exact(z):
    rng = np.random.default_rng(5)
    frames, want = [], []
    for ts in (1, 2, 4, 8, 12):
        for trial in range(4):
            n = int(rng.integers(1, 40000))
            a = rng.poisson(0.5, n * ts).astype(np.uint8)
            if trial == 0:
                a[:] = 3
            d = a.tobytes()
            for shuffle in ("bit", "byte", "none"):
                split = bool(rng.integers(0, 2))
                frames.append(blosc_frame(d, ts, int(rng.choice([8, 64, 1000, 4096])) * ts, shuffle, split))
                want.append(d)
            frames.append(blosc_frame(d, ts, 700 * ts, raw_streams=True))
            want.append(d)
            frames.append(blosc_frame(d, ts, 700 * ts, memcpy=True))
            want.append(d)
    for got, w in zip(_decode(frames), want):
        assert got == w


def test_malformed_streams_are_refused_without_a_fault(z):
    data = b"abcd" * 400
    fr = bytearray(blosc_frame(data, 1, len(data), "none", split=False))
    stream0 = 16 + 4 + 4                           # header, one block start, the stream's size
    assert fr[stream0] >> 4 == 4                   # 4 literals, then the match offset
    bad_offset = bytearray(fr)
    bad_offset[stream0 + 5:stream0 + 7] = b"\xff\xff"   # points before the start of the output
    cut = bytearray(fr)
    struct.pack_into("<i", cut, 20, struct.unpack_from("<i", fr, 20)[0] - 3)   # the stream ends early
    for bad in (bytes(bad_offset), bytes(cut)):
        with pytest.raises(ValueError):
            _decode([bad])
    assert _decode([bytes(fr)])[0] == data        # the context is intact
    with pytest.raises(ValueError):               # a header that claims more than the frame holds
        _decode([bytes(fr[:40])])


def test_chunks_to_csr_and_store_reader(z, tmp_path):
    from scarf_gb300 import kernels as K
    from scarf_gb300.zarr_io import read_counts_csr
    meta = json.loads(str(z["rna_zarray"]))
    n, g = meta["shape"]
    cr, cc = meta["chunks"]
    last = int(z["rna_last_chunk"])
    # a store holding the first and last chunk of the reference's RNA counts (the others missing: zeros)
    d = tmp_path / "RNA" / "counts"
    d.mkdir(parents=True)
    (d / ".zarray").write_text(json.dumps(meta))
    (d / "0.0").write_bytes(z["rna_0_0"].tobytes())
    (d / f"0.{last}").write_bytes(z[f"rna_0_{last}"].tobytes())
    dense = np.zeros((n, g), dtype=np.uint32)
    dense[:, :cc] = blosc.decode_chunk(z["rna_0_0"].tobytes(), (cr, cc), "<u4")[:n]
    dense[:, last * cc:] = blosc.decode_chunk(z[f"rna_0_{last}"].tobytes(), (cr, cc), "<u4")[:n, :g - last * cc]
    want = sp.csr_matrix(dense.astype(np.int64))
    want.sort_indices()
    ip, ind, dat, ng = read_counts_csr(str(tmp_path), "RNA/counts")
    assert ng == g
    assert np.array_equal(ip.cpu().numpy(), want.indptr)
    assert np.array_equal(ind.cpu().numpy(), want.indices)
    assert np.array_equal(dat.cpu().numpy(), want.data)
    # a band with a ragged row count and an offset indptr
    band = torch.zeros((last + 1) * cr * cc, dtype=torch.int32, device="cuda")
    band[:cr * cc] = torch.from_numpy(blosc.decode_chunk(z["rna_0_0"].tobytes(), (cr, cc), "<u4")
                                      .astype(np.int32).reshape(-1)).cuda()
    ip2, ind2, dat2 = K.chunks_to_csr(band, 300, cr, cc, g, indptr_base=17)
    w2 = sp.csr_matrix(dense[:300, :cc].astype(np.int64), shape=(300, g))
    assert np.array_equal(ip2.cpu().numpy() - 17, w2.indptr)
    assert np.array_equal(ind2.cpu().numpy(), w2.indices) and np.array_equal(dat2.cpu().numpy(), w2.data)


def test_datastore_from_zarr(z, tmp_path):
    from scarf_gb300.datastore import DataStore
    meta = json.loads(str(z["rna_zarray"]))
    ids_meta = json.loads(str(z["ids_zarray"]))
    n, g = meta["shape"]
    (tmp_path / "RNA" / "counts").mkdir(parents=True)
    (tmp_path / "RNA" / "counts" / ".zarray").write_text(json.dumps(meta))
    (tmp_path / "RNA" / "counts" / "0.0").write_bytes(z["rna_0_0"].tobytes())
    (tmp_path / "cellData" / "ids").mkdir(parents=True)
    (tmp_path / "cellData" / "ids" / ".zarray").write_text(json.dumps(ids_meta))
    (tmp_path / "cellData" / "ids" / "0").write_bytes(z["cell_ids_0"].tobytes())
    ds = DataStore.from_zarr(str(tmp_path))
    want_ids = np.frombuffer(blosc.decompress(z["cell_ids_0"].tobytes()), dtype=ids_meta["dtype"])[:n]
    assert np.array_equal(ds.cells.fetch_all("ids"), want_ids)
    dense = blosc.decode_chunk(z["rna_0_0"].tobytes(), tuple(meta["chunks"]), "<u4")[:n]
    got = sp.csr_matrix((ds.RNA.data, ds.RNA.indices, ds.RNA.indptr), shape=(n, g))
    assert np.array_equal(got[:, :dense.shape[1]].toarray(), dense.astype(np.int64))
    assert got[:, dense.shape[1]:].nnz == 0
