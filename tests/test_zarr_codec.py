"""The oracle's restatement of scarf's zarr chunk codec (Blosc1 frames, LZ4
blocks, bit and byte shuffle; scarf/writers.py:58-89, :164-204), pinned on the
reference's own test store and exercised on frames of every layout."""
import hashlib
import json
import os

import numpy as np
import pytest

from helpers import blosc_frame, lz4_compress
from oracle import blosc


@pytest.fixture(scope="module")
def z(golden_dir):
    return np.load(os.path.join(golden_dir, "zarr_chunks.npz"))


def test_adt_chunk_decodes_to_the_reference_cell_totals(z):
    # the ADT matrix is one chunk: its decoded per-cell totals and non-zero
    # counts are the reference's assay2_nCounts / assay2_nFeatures
    ids_meta = json.loads(str(z["ids_zarray"]))
    adt_meta = json.loads(str(z["adt_zarray"]))
    n = ids_meta["shape"][0]
    ids = np.frombuffer(blosc.decompress(z["cell_ids_0"].tobytes()), dtype=ids_meta["dtype"])[:n]
    pos = {v: i for i, v in enumerate(ids)}
    sel = np.array([pos[v] for v in z["csv_ids"]])
    adt = blosc.decode_chunk(z["adt_0_0"].tobytes(), tuple(adt_meta["chunks"]), "<u4")[:n, :adt_meta["shape"][1]]
    assert np.array_equal(adt.sum(1)[sel], z["csv_adt_ncounts"])
    assert np.array_equal((adt > 0).sum(1)[sel], z["csv_adt_nfeatures"])
    assert all(s.endswith("-1") for s in ids)                     # readable cell barcodes (byte shuffle)


def test_rna_chunks_match_the_pinned_decoding(z):
    # when the fixture was made, the oracle decoded all 37 RNA chunks and its
    # per-cell totals equalled the reference's RNA_nCounts / RNA_nFeatures
    ids_meta = json.loads(str(z["ids_zarray"]))
    ids = np.frombuffer(blosc.decompress(z["cell_ids_0"].tobytes()), dtype=ids_meta["dtype"])
    pos = {v: i for i, v in enumerate(ids)}
    sel = np.array([pos[v] for v in z["csv_ids"]])
    assert np.array_equal(z["rna_totals_all_chunks"][sel], z["csv_rna_ncounts"])
    assert np.array_equal(z["rna_nnz_all_chunks"][sel], z["csv_rna_nfeatures"])
    meta = json.loads(str(z["rna_zarray"]))
    last = int(z["rna_last_chunk"])
    for key in ("rna_0_0", f"rna_0_{last}", "adt_0_0", "cell_ids_0"):
        raw = blosc.decompress(z[key].tobytes())
        assert hashlib.sha256(raw).hexdigest() == str(z[f"sha256_{key}"])
    h = blosc.parse_header(z["rna_0_0"].tobytes())
    assert h["flags"] & blosc.FLAG_BITSHUFFLE and not h["flags"] & blosc.FLAG_NOSPLIT and h["typesize"] == 4
    c = blosc.decode_chunk(z[f"rna_0_{last}"].tobytes(), tuple(meta["chunks"]), "<u4")
    w = meta["shape"][1] - last * meta["chunks"][1]
    assert not c[:, w:].any() and not c[meta["shape"][0]:].any()   # padding past the array is zero


@pytest.mark.parametrize("ts", [1, 2, 4, 8, 12])
def test_frames_of_every_layout_round_trip(ts):
    rng = np.random.default_rng(ts)
    for trial in range(6):
        n = int(rng.integers(1, 6000))
        a = rng.poisson(0.4, n * ts).astype(np.uint8)
        if trial == 0:
            a[:] = 9                                   # long overlapping matches
        d = a.tobytes()
        for shuffle in ("bit", "byte", "none"):
            for split in (True, False):
                bs = int(rng.choice([8, 64, 1000])) * ts
                assert blosc.decompress(blosc_frame(d, ts, bs, shuffle, split)) == d
        assert blosc.decompress(blosc_frame(d, ts, 512 * ts, raw_streams=True)) == d
        assert blosc.decompress(blosc_frame(d, ts, 512 * ts, memcpy=True)) == d


def test_lz4_rejects_a_bad_offset():
    good = lz4_compress(b"abcd" * 40)
    assert blosc.lz4_block_decompress(good, 160) == b"abcd" * 40
    with pytest.raises(ValueError):
        blosc.lz4_block_decompress(bytes([0x04, 9, 0, 0]), 8)   # a match before any output
