"""CPU restatement of the chunk codec of scarf's zarr stores (test
infrastructure: the oracle for the GPU decoder).

scarf writes its count matrices with ``create_zarr_dataset``
(scarf/writers.py:58-89): zarr v2 arrays compressed by numcodecs' Blosc with
``cname='lz4'``, ``clevel=5`` and ``shuffle=Blosc.BITSHUFFLE`` (dense ``<u4``
counts, chunks of 1000 x 1000 cells x genes, scarf/writers.py:164-204); string
arrays such as feature ids use byte shuffle. numcodecs wraps c-blosc 1.x
(pinned below 0.16 in scarf's requirements); the three published formats it
uses are restated here:

* Blosc1 frame: a 16-byte header -- version, LZ version, flags, type size
  (one byte each), then uncompressed bytes, block size and compressed bytes
  (little-endian uint32) -- and, unless the frame is a plain copy (flag
  0x02), one int32 start offset per block. Flags: 0x01 byte shuffle, 0x04
  bit shuffle, 0x10 blocks not split, bits 5-7 the codec (1 = LZ4). A block
  of a frame without 0x10 is split into ``typesize`` streams (one per byte of
  an element) unless it is the last, shorter block; each stream is an int32
  compressed size and then LZ4 data, or the raw bytes when that size equals
  the stream's length.
* LZ4 block: sequences of a token (high nibble literal length, low nibble
  match length - 4, 15 meaning "more bytes follow, each added, until one is
  below 255"), the literals, then a little-endian 16-bit offset back into the
  output and the match (which may overlap its own output); the last sequence
  has literals only.
* bit shuffle (bitshuffle's bit-plane transpose) of a block of n elements of
  ``typesize`` bytes: for n rounded down to a multiple of 8, bit j of byte b
  of element e sits in bit-plane 8 b + j, at bit e of that plane (least
  significant bit first); the remaining n % 8 elements are stored as they
  are. Byte shuffle stores byte b of every element together.

Pinned on the reference's own chunks (tests/golden/zarr_chunks.npz, made by
tests/golden/make_golden.py from scarf/tests/datasets/1K_pbmc_citeseq.zarr):
the feature-id strings decode to readable gene names and the decoded counts
to the reference's cell and feature totals.
"""
from __future__ import annotations

import struct
from typing import List, Tuple

import numpy as np

FLAG_SHUFFLE = 0x01
FLAG_MEMCPYED = 0x02
FLAG_BITSHUFFLE = 0x04
FLAG_NOSPLIT = 0x10
CODEC_LZ4 = 1


def lz4_block_decompress(src: bytes, out_len: int) -> bytes:
    """Decode one LZ4 block (published block format) of known output length."""
    out = bytearray(out_len)
    ip = 0
    op = 0
    n = len(src)
    while ip < n:
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
        out[op:op + lit] = src[ip:ip + lit]
        ip += lit
        op += lit
        if ip >= n:                      # the last sequence has literals only
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
            raise ValueError("lz4: bad match offset")
        start = op - off
        if off >= mlen:
            out[op:op + mlen] = out[start:start + mlen]
        else:                            # overlapping match: repeats the last `off` bytes
            for i in range(mlen):
                out[op + i] = out[start + i]
        op += mlen
    if op != out_len:
        raise ValueError(f"lz4: decoded {op} bytes, expected {out_len}")
    return bytes(out)


def bitunshuffle(buf: bytes, typesize: int) -> bytes:
    """Inverse of the bit-plane transpose of one block."""
    n = len(buf) // typesize
    n8 = n - n % 8
    if n8 == 0:
        return bytes(buf)
    planes = np.frombuffer(buf[:n8 * typesize], dtype=np.uint8).reshape(typesize * 8, n8 // 8)
    bits = np.unpackbits(planes, axis=1, bitorder="little")          # [8 b + j, e]
    bits = bits.reshape(typesize, 8, n8).transpose(2, 0, 1)          # [e, b, j]
    elems = np.packbits(bits, axis=2, bitorder="little").reshape(-1)  # byte b of element e
    return elems.tobytes() + bytes(buf[n8 * typesize:])


def byteunshuffle(buf: bytes, typesize: int) -> bytes:
    n = len(buf) // typesize
    body = np.frombuffer(buf[:n * typesize], dtype=np.uint8).reshape(typesize, n).T.reshape(-1)
    return body.tobytes() + bytes(buf[n * typesize:])


def parse_header(frame: bytes) -> dict:
    ver, verlz, flags, typesize = frame[0], frame[1], frame[2], frame[3]
    nbytes, blocksize, cbytes = struct.unpack_from("<III", frame, 4)
    nblocks = (nbytes + blocksize - 1) // blocksize if blocksize else 0
    memcpyed = bool(flags & FLAG_MEMCPYED)
    starts = [] if memcpyed else list(struct.unpack_from(f"<{nblocks}i", frame, 16))
    return dict(version=ver, versionlz=verlz, flags=flags, typesize=typesize, nbytes=nbytes, blocksize=blocksize,
                cbytes=cbytes, nblocks=nblocks, starts=starts, memcpyed=memcpyed, codec=flags >> 5)


def block_streams(hdr: dict, b: int) -> Tuple[int, int]:
    """(uncompressed bytes of block b, number of streams it is split into)."""
    bs = hdr["blocksize"]
    last = hdr["nbytes"] - b * bs if b == hdr["nblocks"] - 1 else bs
    split = not (hdr["flags"] & FLAG_NOSPLIT) and last == bs
    return last, (hdr["typesize"] if split else 1)


def decompress(frame: bytes) -> bytes:
    """One Blosc1 frame (LZ4 codec, with or without shuffles) to its bytes."""
    h = parse_header(frame)
    if h["memcpyed"]:
        return bytes(frame[16:16 + h["nbytes"]])
    if h["codec"] != CODEC_LZ4:
        raise NotImplementedError("only the LZ4 codec is restated")
    out = bytearray()
    for b in range(h["nblocks"]):
        blen, ns = block_streams(h, b)
        slen = blen // ns
        ip = h["starts"][b]
        parts: List[bytes] = []
        for _ in range(ns):
            csize = struct.unpack_from("<i", frame, ip)[0]
            ip += 4
            if csize == slen:
                parts.append(bytes(frame[ip:ip + csize]))
            else:
                parts.append(lz4_block_decompress(frame[ip:ip + csize], slen))
            ip += csize
        blk = b"".join(parts)
        if h["flags"] & FLAG_BITSHUFFLE:
            blk = bitunshuffle(blk, h["typesize"])
        elif h["flags"] & FLAG_SHUFFLE:
            blk = byteunshuffle(blk, h["typesize"])
        out += blk
    return bytes(out)


def decode_chunk(frame: bytes, shape, dtype) -> np.ndarray:
    return np.frombuffer(decompress(frame), dtype=dtype).reshape(shape)
