"""Shared helpers of the test suite (seeded inputs, device transfers)."""
import numpy as np
import scipy.sparse as sp


def small_counts(n_cells=1500, n_genes=3000, n_clusters=6, seed=0, empty_rows=(3, 700)):
    """Seeded NB-like CSR counts (numpy, fast) with a few empty rows."""
    rng = np.random.default_rng(seed)
    mu = np.exp(rng.normal(-1.0, 1.5, n_genes))
    prog = np.ones((n_clusters, n_genes))
    for c in range(n_clusters):
        prog[c, rng.choice(n_genes, 60, replace=False)] = rng.uniform(2, 4, 60)
    p = mu * prog
    p /= p.sum(1, keepdims=True)
    lab = rng.integers(0, n_clusters, n_cells)
    lib = np.exp(np.log(1500) + 0.4 * rng.normal(size=n_cells))
    lam = lib[:, None] * p[lab] * rng.gamma(2.0, 0.5, size=(n_cells, n_genes))
    cnt = rng.poisson(lam).astype(np.int32)
    for r in empty_rows:
        if r < n_cells:
            cnt[r] = 0
    m = sp.csr_matrix(cnt)
    m.sort_indices()
    return m.indptr.astype(np.int64), m.indices.astype(np.int32), m.data.astype(np.int32), n_genes, lab


def top_var_genes(indptr, indices, data, n_genes, n_top):
    n = len(indptr) - 1
    lib = np.add.reduceat(data.astype(np.int64), indptr[:-1]) if len(data) else np.zeros(n)
    lib[np.diff(indptr) == 0] = 0
    lib = np.maximum(lib, 1)
    rows = np.repeat(np.arange(n), np.diff(indptr))
    x = np.log1p(1000.0 * data / lib[rows])
    s1 = np.bincount(indices, weights=x, minlength=n_genes)
    s2 = np.bincount(indices, weights=x * x, minlength=n_genes)
    var = s2 / n - (s1 / n) ** 2
    return np.sort(np.argsort(-var, kind="stable")[:n_top])


def clustered_points(n, d, n_clusters=8, seed=0, spread=0.6, dup=()):
    rng = np.random.default_rng(seed)
    centers = rng.normal(0, 4, size=(n_clusters, d))
    lab = rng.integers(0, n_clusters, n)
    x = centers[lab] + spread * rng.normal(size=(n, d))
    for a, b in dup:
        x[b] = x[a]
    return x.astype(np.float32)


def umap_graph(n, d, n_clusters, k, seed):
    """Clustered points, their labels and the fused UMAP graph of their exact
    kNN (oracle smoothing + fuzzy union) as COO arrays (head, tail, weight)."""
    import oracle
    rng = np.random.default_rng(seed)
    centers = rng.normal(0, 6, size=(n_clusters, d))
    lab = rng.integers(0, n_clusters, n)
    x = (centers[lab] + rng.normal(size=(n, d))).astype(np.float32)
    ki, kd = oracle.exact_knn(x, x, k + 1)
    fi, fd, _ = oracle.fix_knn_query(ki, kd.astype(np.float32), np.arange(n))
    edges, w = oracle.smoothen_dists(fi.astype(np.uint64), fd.astype(np.float64), 1.0, 1.5, 1000)
    import scipy.sparse as sp
    g = sp.csr_matrix((w, (edges[:, 0].astype(np.int64), edges[:, 1].astype(np.int64))), shape=(n, n))
    u = oracle.fuzzy_simplicial_set(g, 1.0).tocsr()
    u.sort_indices()
    u = u.tocoo()
    return x, lab, g, u.row.astype(np.int64), u.col.astype(np.int64), u.data


def embedding_purity(y, lab, k=10):
    """Fraction of each point's k nearest embedded neighbours in its cluster."""
    d = ((y[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d, np.inf)
    nn = np.argsort(d, axis=1)[:, :k]
    return float((lab[nn] == lab[:, None]).mean())


def multirank_worker(rank, ws, port, q):
    """One rank of a CPU (gloo) process group: reports bench.max_over_ranks of
    a rank-dependent step time."""
    import os
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    q.put((rank, bench.max_over_ranks(10.0 + rank, torch.device("cpu")), bench.dist_env()))
    dist.barrier()
    dist.destroy_process_group()


# ---- Blosc1 / LZ4 / bit-shuffle frames for decoder tests (the encoder side of
# the published formats, small and simple: greedy LZ4 matching, no search) ----
def lz4_compress(data: bytes, min_match: int = 4) -> bytes:
    """A valid LZ4 block of ``data``: greedy matches found through a table of
    the last position of each 4-byte prefix (offsets < 65536, overlapping
    matches allowed), the last 5 bytes as literals as the format requires."""
    out = bytearray()
    n = len(data)
    table = {}
    i = anchor = 0

    def length_bytes(v):
        while v >= 255:
            out.append(255)
            v -= 255
        out.append(v)

    def emit(lit_start, lit_end, off=None, mlen=0):
        lit = lit_end - lit_start
        tok_l = min(lit, 15)
        tok_m = 0 if off is None else min(mlen - 4, 15)
        out.append((tok_l << 4) | tok_m)
        if lit >= 15:
            length_bytes(lit - 15)
        out.extend(data[lit_start:lit_end])
        if off is not None:
            out.extend((off & 255, off >> 8))
            if mlen - 4 >= 15:
                length_bytes(mlen - 4 - 15)

    while i + 12 <= n:
        key = data[i:i + 4]
        j = table.get(key)
        table[key] = i
        if j is not None and i - j < 65536:
            m = 4
            while i + m < n - 5 and data[j + m] == data[i + m]:
                m += 1
            if m >= min_match:
                emit(anchor, i, i - j, m)
                i += m
                anchor = i
                continue
        i += 1
    emit(anchor, n)
    return bytes(out)


def bitshuffle(buf: bytes, typesize: int) -> bytes:
    n = len(buf) // typesize
    n8 = n - n % 8
    if n8 == 0:
        return bytes(buf)
    e = np.frombuffer(buf[:n8 * typesize], dtype=np.uint8).reshape(n8, typesize)
    bits = np.unpackbits(e, axis=1, bitorder="little").reshape(n8, typesize, 8)   # [e, b, j]
    planes = bits.transpose(1, 2, 0).reshape(typesize * 8, n8)                   # [8 b + j, e]
    return np.packbits(planes, axis=1, bitorder="little").tobytes() + bytes(buf[n8 * typesize:])


def byteshuffle(buf: bytes, typesize: int) -> bytes:
    n = len(buf) // typesize
    body = np.frombuffer(buf[:n * typesize], dtype=np.uint8).reshape(n, typesize).T.reshape(-1)
    return body.tobytes() + bytes(buf[n * typesize:])


def blosc_frame(data: bytes, typesize: int, blocksize: int, shuffle: str = "bit", split: bool = True,
                raw_streams: bool = False, memcpy: bool = False) -> bytes:
    """A Blosc1 frame (LZ4 codec) of ``data`` in the layout c-blosc 1.x writes."""
    import struct
    flags = (1 << 5) | {"bit": 0x04, "byte": 0x01, "none": 0}[shuffle] | (0 if split else 0x10)
    nbytes = len(data)
    if memcpy:
        hdr = struct.pack("<BBBBIII", 2, 1, flags | 0x02, typesize, nbytes, blocksize, 16 + nbytes)
        return hdr + data
    nblocks = -(-nbytes // blocksize)
    body = bytearray()
    starts = []
    base = 16 + 4 * nblocks
    for b in range(nblocks):
        blk = data[b * blocksize:(b + 1) * blocksize]
        if shuffle == "bit":
            blk = bitshuffle(blk, typesize)
        elif shuffle == "byte":
            blk = byteshuffle(blk, typesize)
        ns = typesize if (split and len(blk) == blocksize) else 1
        starts.append(base + len(body))
        sl = len(blk) // ns
        for k in range(ns):
            s = blk[k * sl:(k + 1) * sl]
            c = s if raw_streams else lz4_compress(s)
            if len(c) >= len(s):
                c = s          # stored raw: the compressed size equals the stream's length
            body += struct.pack("<i", len(c)) + c
    hdr = struct.pack("<BBBBIII", 2, 1, flags, typesize, nbytes, blocksize, base + len(body))
    return hdr + struct.pack(f"<{nblocks}i", *starts) + bytes(body)


def lz4_check_block(src: bytes, out_len: int) -> None:
    """Raise unless ``src`` is an LZ4 block that follows the format's
    end-of-block rules: the last sequence is literals only, the last 5 bytes
    of the output are literals, no match starts within the last 12 bytes,
    offsets point inside the output and the sequences decode to ``out_len``
    bytes."""
    ip = op = 0
    n = len(src)
    while True:
        if ip >= n:
            raise ValueError("lz4: missing last sequence")
        token = src[ip]
        ip += 1
        lit = token >> 4
        if lit == 15:
            while True:
                b = src[ip]
                ip += 1
                lit += b
                if b != 255:
                    break
        ip += lit
        op += lit
        if ip > n:
            raise ValueError("lz4: literals past the end")
        if ip == n:
            if token & 15:
                raise ValueError("lz4: last token announces a match")
            break
        off = src[ip] | (src[ip + 1] << 8)
        ip += 2
        mlen = (token & 15) + 4
        if (token & 15) == 15:
            while True:
                b = src[ip]
                ip += 1
                mlen += b
                if b != 255:
                    break
        if off == 0 or off > op:
            raise ValueError("lz4: offset outside the output")
        if op + 12 > out_len:
            raise ValueError("lz4: a match starts within the last 12 bytes")
        op += mlen
        if op > out_len - 5:
            raise ValueError("lz4: a match reaches into the last 5 bytes")
    if op != out_len:
        raise ValueError(f"lz4: {op} bytes, expected {out_len}")


def check_frame(frame: bytes) -> dict:
    """Check a Blosc1 frame's header and every LZ4 stream of its blocks
    against the format rules; return the parsed header."""
    import struct
    version, vlz, flags, ts, nbytes, bsize, cbytes = struct.unpack_from("<BBBBIII", frame, 0)
    assert cbytes == len(frame), (cbytes, len(frame))
    assert version == 2 and vlz == 1 and (flags >> 5) == 1
    if nbytes:
        nb = -(-nbytes // bsize)
        starts = struct.unpack_from(f"<{nb}i", frame, 16)
        for b, st in enumerate(starts):
            blen = min(bsize, nbytes - b * bsize)
            nsplit = ts if (not (flags & 0x10) and blen == bsize) else 1
            pos = st
            for _ in range(nsplit):
                cs = struct.unpack_from("<i", frame, pos)[0]
                pos += 4
                slen = blen // nsplit
                if cs != slen:
                    lz4_check_block(frame[pos:pos + cs], slen)
                pos += cs
    return {"flags": flags, "typesize": ts, "nbytes": nbytes, "blocksize": bsize}
