// f2: decoding scarf's zarr chunks on the device. scarf writes its count
// matrices with create_zarr_dataset (scarf/writers.py:58-89, :164-204):
// numcodecs Blosc frames (c-blosc 1.x format), LZ4 codec, bit shuffle for the
// dense uint32 counts (byte shuffle for string arrays). The formats:
//
// * Blosc1 frame: 16-byte header (version, LZ version, flags, type size;
//   uncompressed bytes, block size, compressed bytes), then one int32 start
//   offset per block unless the frame is a plain copy (flag 0x02). Flags: 0x01
//   byte shuffle, 0x04 bit shuffle, 0x10 blocks not split, bits 5-7 the codec
//   (1 = LZ4). A full block of a frame without 0x10 is split into `typesize`
//   streams; each stream is an int32 compressed size and LZ4 data, or raw
//   bytes when that size equals the stream's length.
// * LZ4 block: tokens (literal length, match length - 4; 15 = more length
//   bytes follow), literals, a 16-bit little-endian match offset.
// * bit shuffle: for n elements rounded down to a multiple of 8, bit j of
//   byte b of element e is bit e (LSB first) of bit-plane 8 b + j; the rest
//   are stored as they are.
//
// The host parses and checks the headers and lists the streams and blocks.
// lz4_stream_kernel: one warp per stream; lane 0 parses the tokens, the warp
// copies literals and matches together (a match that overlaps its own output
// repeats the last `offset` bytes: byte i of it is out[op - off + i % off]).
// Every read and write is bounds-checked: a malformed stream raises an error
// flag instead of touching memory outside its buffers.
// bitunshuffle_kernel: a warp per 32 elements of a block; lane l holds the
// 32-bit word of bit-plane l, and one ballot per element gathers its bits.
#include "common.cuh"

#include <cstring>

namespace {

struct Stream {
  int64_t src;    // offset of the compressed bytes in the frame buffer
  int64_t dst;    // offset of the output in the destination buffer
  int32_t csize;  // compressed bytes
  int32_t len;    // decoded bytes
  int32_t raw;    // stored uncompressed
  int32_t to_tmp; // output goes to the shuffle staging buffer
};

struct Block {
  int64_t off;    // offset of the block in the output (and in the staging buffer)
  int32_t len;
  int32_t typesize;
  int32_t bit;    // 1: bit shuffle, 0: byte shuffle
};

__global__ void lz4_stream_kernel(const uint8_t* __restrict__ src, const Stream* __restrict__ streams, int n_streams,
                                  uint8_t* __restrict__ out, uint8_t* __restrict__ tmp, int* __restrict__ err) {
  const int si = blockIdx.x;
  if (si >= n_streams) return;
  const Stream s = streams[si];
  const uint8_t* in = src + s.src;
  uint8_t* o = (s.to_tmp ? tmp : out) + s.dst;
  const int lane = threadIdx.x;
  if (s.raw) {
    for (int i = lane; i < s.len; i += 32) o[i] = in[i];
    return;
  }
  int ip = 0, op = 0;
  bool bad = false;
  while (true) {
    int lit = 0, moff = 0, mlen = 0, nip = 0;
    int code = 0;  // 0 ok, 1 last sequence, 2 malformed
    if (lane == 0) {
      int p = ip;
      if (p >= s.csize) {
        code = 2;
      } else {
        const int token = in[p++];
        lit = token >> 4;
        if (lit == 15) {
          int b;
          do {
            if (p >= s.csize) { code = 2; break; }
            b = in[p++];
            lit += b;
          } while (b == 255);
        }
        if (code == 0 && (p + lit > s.csize || op + lit > s.len)) code = 2;
        const int lp = p;
        p += lit;
        if (code == 0 && p == s.csize) {
          code = 1;
        } else if (code == 0) {
          if (p + 2 > s.csize) {
            code = 2;
          } else {
            moff = in[p] | (in[p + 1] << 8);
            p += 2;
            mlen = (token & 15) + 4;
            if ((token & 15) == 15) {
              int b;
              do {
                if (p >= s.csize) { code = 2; break; }
                b = in[p++];
                mlen += b;
              } while (b == 255);
            }
            if (code == 0 && (moff == 0 || moff > op + lit || op + lit + mlen > s.len)) code = 2;
          }
        }
        nip = p;
        lit = (code == 2) ? 0 : lit;
        ip = lp;  // literals start here
      }
    }
    code = __shfl_sync(0xffffffffu, code, 0);
    lit = __shfl_sync(0xffffffffu, lit, 0);
    const int lp = __shfl_sync(0xffffffffu, ip, 0);
    if (code == 2) {
      bad = true;
      break;
    }
    for (int i = lane; i < lit; i += 32) o[op + i] = in[lp + i];
    op += lit;
    if (code == 1) break;
    moff = __shfl_sync(0xffffffffu, moff, 0);
    mlen = __shfl_sync(0xffffffffu, mlen, 0);
    nip = __shfl_sync(0xffffffffu, nip, 0);
    __syncwarp();  // the bytes a match repeats are written
    for (int i = lane; i < mlen; i += 32) o[op + i] = __ldcg(o + op - moff + (i % moff));
    __syncwarp();
    op += mlen;
    ip = nip;
  }
  if (lane == 0 && (bad || op != s.len)) atomicCAS(err, 0, 1);
}

// one warp per 32 elements of a bit-shuffled block (global work index over
// all blocks given as a prefix of 32-element groups)
__global__ void bitunshuffle_kernel(const uint8_t* __restrict__ tmp, uint8_t* __restrict__ out,
                                    const Block* __restrict__ blocks, const int64_t* __restrict__ group_start,
                                    int n_blocks, int64_t n_groups) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (gw >= n_groups) return;
  int lo = 0, hi = n_blocks - 1;  // the block holding group gw
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (group_start[mid] <= gw) lo = mid;
    else hi = mid - 1;
  }
  const Block b = blocks[lo];
  const int ts = b.typesize;
  const int64_t n = b.len / ts;
  const int64_t n8 = n - n % 8;
  const int64_t plane_bytes = n8 / 8;
  const int64_t e0 = (gw - group_start[lo]) * 32;  // first element of this group
  const uint8_t* in = tmp + b.off;
  uint8_t* o = out + b.off;
  // the elements past the last multiple of 8, and the bytes past the last
  // whole element, are stored as they are
  for (int64_t i = max(e0, n8) * ts + lane; i < min(n, e0 + 32) * ts; i += 32) o[i] = in[i];
  if (e0 + 32 >= n)
    for (int64_t i = n * ts + lane; i < b.len; i += 32) o[i] = in[i];
  if (e0 >= n8) return;
  const int cnt = int(n8 - e0 < 32 ? n8 - e0 : 32);
  for (int g = 0; g < (8 * ts + 31) / 32; ++g) {
    const int p = 32 * g + lane;  // this lane's bit-plane
    uint32_t word = 0;
    if (p < 8 * ts) {
      const uint8_t* pl = in + int64_t(p) * plane_bytes + e0 / 8;
      for (int q = 0; q < (cnt + 7) / 8; ++q) word |= uint32_t(pl[q]) << (8 * q);
    }
    uint32_t mine = 0;
    for (int i = 0; i < cnt; ++i) {
      const uint32_t m = __ballot_sync(0xffffffffu, (word >> i) & 1u);
      if (lane == i) mine = m;
    }
    // lane i: bytes 4g .. 4g+3 of element e0 + i
    if (lane < cnt) {
      for (int q = 0; q < 4 && 4 * g + q < ts; ++q) o[(e0 + lane) * ts + 4 * g + q] = uint8_t(mine >> (8 * q));
    }
  }
}

__global__ void byteunshuffle_kernel(const uint8_t* __restrict__ tmp, uint8_t* __restrict__ out, Block b) {
  const int ts = b.typesize;
  const int64_t n = b.len / ts;
  const uint8_t* in = tmp + b.off;
  uint8_t* o = out + b.off;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < b.len; i += int64_t(gridDim.x) * blockDim.x) {
    if (i < n * ts) {
      const int64_t e = i / ts;
      const int bb = int(i - e * ts);
      o[i] = in[int64_t(bb) * n + e];
    } else {
      o[i] = in[i];
    }
  }
}

uint32_t rd32(const uint8_t* p) { return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24); }

}  // namespace

extern "C" int sg_blosc_decode(sg_handle* h, const uint8_t* frames, const int64_t* frame_offsets, int32_t n_frames,
                               void* out, int64_t out_bytes, const int64_t* out_starts, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(n_frames >= 0 && (n_frames == 0 || (frames && frame_offsets && out && out_starts)),
         "sg_blosc_decode: null pointer argument");
  if (n_frames == 0) return SG_OK;
  std::vector<Stream> streams;
  std::vector<Block> bit_blocks, byte_blocks;
  std::vector<int64_t> group_start;
  int64_t groups = 0;
  const int64_t total_in = frame_offsets[n_frames] - frame_offsets[0];
  const int64_t total_out = out_bytes;
  SG_ARG(total_in >= 0 && total_out >= 0, "sg_blosc_decode: offsets must not decrease");
  for (int f = 0; f < n_frames; ++f) {
    const uint8_t* fr = frames + frame_offsets[f];
    const int64_t flen = frame_offsets[f + 1] - frame_offsets[f];
    const int64_t fin = frame_offsets[f] - frame_offsets[0];
    const int64_t fout = out_starts[f];
    SG_ARG(flen >= 16, "sg_blosc_decode: frame %d shorter than its header", f);
    const int version = fr[0], flags = fr[2], ts = fr[3];
    const int64_t nbytes = rd32(fr + 4), blocksize = rd32(fr + 8), cbytes = rd32(fr + 12);
    SG_ARG(version >= 1 && version <= 3, "sg_blosc_decode: frame %d: not a Blosc1 frame (version %d)", f, version);
    SG_ARG(cbytes <= flen, "sg_blosc_decode: frame %d: %lld compressed bytes in a buffer of %lld", f,
           (long long)cbytes, (long long)flen);
    SG_ARG(fout >= 0 && fout + nbytes <= out_bytes,
           "sg_blosc_decode: frame %d decodes to %lld bytes at offset %lld, past the %lld-byte output", f,
           (long long)nbytes, (long long)fout, (long long)out_bytes);
    SG_ARG(ts >= 1, "sg_blosc_decode: frame %d: type size 0", f);
    if (nbytes == 0) continue;
    if (flags & 0x02) {  // plain copy
      SG_ARG(16 + nbytes <= cbytes, "sg_blosc_decode: frame %d: short plain copy", f);
      int64_t done = 0;
      while (done < nbytes) {  // raw streams of at most 2^30 bytes
        const int32_t len = int32_t(std::min<int64_t>(nbytes - done, int64_t(1) << 30));
        streams.push_back({fin + 16 + done, fout + done, len, len, 1, 0});
        done += len;
      }
      continue;
    }
    SG_ARG((flags >> 5) == 1, "sg_blosc_decode: frame %d: codec %d (only LZ4 is supported)", f, flags >> 5);
    SG_ARG(!(flags & 0x08), "sg_blosc_decode: frame %d: delta filter is not supported", f);
    SG_ARG(blocksize > 0 && blocksize < (int64_t(1) << 31), "sg_blosc_decode: frame %d: bad block size", f);
    const int64_t nblocks = (nbytes + blocksize - 1) / blocksize;
    SG_ARG(16 + 4 * nblocks <= cbytes, "sg_blosc_decode: frame %d: block table past the frame", f);
    const bool shuffled = (flags & 0x05) != 0;
    for (int64_t b = 0; b < nblocks; ++b) {
      const int64_t blen = b == nblocks - 1 ? nbytes - b * blocksize : blocksize;
      const int nsplit = (!(flags & 0x10) && blen == blocksize) ? ts : 1;
      SG_ARG(blen % nsplit == 0, "sg_blosc_decode: frame %d: block not divisible into streams", f);
      const int64_t slen = blen / nsplit;
      int64_t ip = int64_t(int32_t(rd32(fr + 16 + 4 * b)));
      for (int k = 0; k < nsplit; ++k) {
        SG_ARG(ip >= 16 && ip + 4 <= cbytes, "sg_blosc_decode: frame %d: stream outside the frame", f);
        const int64_t cs = int64_t(int32_t(rd32(fr + ip)));
        ip += 4;
        SG_ARG(cs > 0 && ip + cs <= cbytes, "sg_blosc_decode: frame %d: stream of %lld bytes outside the frame", f,
               (long long)cs);
        streams.push_back({fin + ip, fout + b * blocksize + k * slen, int32_t(cs), int32_t(slen),
                           cs == slen ? 1 : 0, shuffled ? 1 : 0});
        ip += cs;
      }
      if (flags & 0x04) {
        bit_blocks.push_back({fout + b * blocksize, int32_t(blen), ts, 1});
        group_start.push_back(groups);
        groups += std::max<int64_t>(1, ((blen / ts) + 31) / 32);
      } else if (flags & 0x01) {
        byte_blocks.push_back({fout + b * blocksize, int32_t(blen), ts, 0});
      }
    }
  }
  const bool need_tmp = !bit_blocks.empty() || !byte_blocks.empty();
  const size_t need = sg::Carver::need(size_t(total_in)) + sg::Carver::need(sizeof(Stream) * streams.size()) +
                      sg::Carver::need(sizeof(Block) * bit_blocks.size() + 8) +
                      sg::Carver::need(sizeof(int64_t) * group_start.size() + 8) +
                      (need_tmp ? sg::Carver::need(size_t(total_out)) : 0) + sg::Carver::need(sizeof(int));
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  uint8_t* d_in = cv.take<uint8_t>(size_t(total_in));
  Stream* d_streams = cv.take<Stream>(streams.size());
  Block* d_blocks = cv.take<Block>(bit_blocks.size() + 1);
  int64_t* d_gs = cv.take<int64_t>(group_start.size() + 1);
  uint8_t* d_tmp = need_tmp ? cv.take<uint8_t>(size_t(total_out)) : nullptr;
  int* err = cv.take<int>(1);
  uint8_t* d_out = static_cast<uint8_t*>(out);
  SG_CUDA(cudaMemcpyAsync(d_in, frames + frame_offsets[0], size_t(total_in), cudaMemcpyHostToDevice, st));
  SG_CUDA(cudaMemcpyAsync(d_streams, streams.data(), sizeof(Stream) * streams.size(), cudaMemcpyHostToDevice, st));
  if (!bit_blocks.empty()) {
    SG_CUDA(cudaMemcpyAsync(d_blocks, bit_blocks.data(), sizeof(Block) * bit_blocks.size(), cudaMemcpyHostToDevice,
                            st));
    SG_CUDA(cudaMemcpyAsync(d_gs, group_start.data(), sizeof(int64_t) * group_start.size(), cudaMemcpyHostToDevice,
                            st));
  }
  SG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  sg::ProfScope prof(h, "blosc", st);
  if (!streams.empty()) {
    lz4_stream_kernel<<<unsigned(streams.size()), 32, 0, st>>>(d_in, d_streams, int(streams.size()), d_out, d_tmp,
                                                              err);
    SG_LAUNCH_CHECK();
  }
  if (groups > 0) {
    bitunshuffle_kernel<<<unsigned(sg::ceil_div(groups * 32, 256)), 256, 0, st>>>(
        d_tmp, d_out, d_blocks, d_gs, int(bit_blocks.size()), groups);
    SG_LAUNCH_CHECK();
  }
  for (const Block& b : byte_blocks) {
    byteunshuffle_kernel<<<unsigned(std::min<int64_t>(sg::ceil_div(b.len, 256), int64_t(h->sm_count) * 8)), 256, 0,
                           st>>>(d_tmp, d_out, b);
    SG_LAUNCH_CHECK();
  }
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (herr) return sg::fail(SG_ERR_ARG, "sg_blosc_decode: a compressed stream is malformed");
  return SG_OK;
}

// ---- dense count chunks -> CSR -------------------------------------------
namespace {

// non-zeros of row r across the band's chunks (a warp per row)
__global__ void chunk_row_count_kernel(const uint32_t* __restrict__ chunks, int64_t n_rows, int cr, int cc,
                                       int64_t n_cols, int64_t* __restrict__ cnt, int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (r >= n_rows) return;
  const int nchunk = int((n_cols + cc - 1) / cc);
  int64_t c = 0;
  bool big = false;
  for (int k = 0; k < nchunk; ++k) {
    const int w = int(min(int64_t(cc), n_cols - int64_t(k) * cc));
    const uint32_t* row = chunks + (int64_t(k) * cr + r) * cc;
    for (int j = lane; j < w; j += 32) {
      const uint32_t v = row[j];
      c += v != 0u;
      big |= v > 0x7fffffffu;
    }
  }
  c = warp_sum_ll(c);
  if (__any_sync(0xffffffffu, big) && lane == 0) atomicCAS(err, 0, 1);
  if (lane == 0) cnt[r] = c;
}

// exclusive scan of cnt into indptr (one CTA of 1024 threads), starting at base
__global__ void __launch_bounds__(1024)
row_scan_kernel(const int64_t* __restrict__ cnt, int64_t n, int64_t base, int64_t* __restrict__ indptr) {
  __shared__ int64_t part[1024];
  const int64_t per = (n + 1023) / 1024;
  const int64_t a = int64_t(threadIdx.x) * per, b = min(n, a + per);
  int64_t s = 0;
  for (int64_t i = a; i < b; ++i) s += cnt[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int64_t run = base + (threadIdx.x ? part[threadIdx.x - 1] : 0);
  for (int64_t i = a; i < b; ++i) {
    indptr[i] = run;
    run += cnt[i];
  }
  if (threadIdx.x == 1023) indptr[n] = base + part[1023];
}

// columns and values of row r in ascending column order (a warp per row,
// ballot compaction of each 32-column group)
__global__ void chunk_row_scatter_kernel(const uint32_t* __restrict__ chunks, int64_t n_rows, int cr, int cc,
                                         int64_t n_cols, const int64_t* __restrict__ indptr, int64_t base,
                                         int64_t capacity, int32_t* __restrict__ ind, int32_t* __restrict__ dat) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (r >= n_rows) return;
  const int nchunk = int((n_cols + cc - 1) / cc);
  int64_t pos = indptr[r] - base;
  const unsigned lt = (1u << lane) - 1u;
  for (int k = 0; k < nchunk; ++k) {
    const int w = int(min(int64_t(cc), n_cols - int64_t(k) * cc));
    const uint32_t* row = chunks + (int64_t(k) * cr + r) * cc;
    for (int j0 = 0; j0 < w; j0 += 32) {
      const int j = j0 + lane;
      const uint32_t v = j < w ? row[j] : 0u;
      const unsigned m = __ballot_sync(0xffffffffu, v != 0u);
      const int64_t at = pos + __popc(m & lt);
      if (v != 0u && at < capacity) {
        ind[at] = int32_t(int64_t(k) * cc + j);
        dat[at] = int32_t(v);
      }
      pos += __popc(m);
    }
  }
}

}  // namespace

extern "C" int sg_chunks_to_csr(sg_handle* h, const uint32_t* chunks, int64_t n_rows, int32_t chunk_rows,
                                int32_t chunk_cols, int64_t n_cols, int64_t indptr_base, int64_t* indptr_out,
                                int32_t* indices_out, int32_t* data_out, int64_t capacity, int64_t* nnz_out,
                                void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(chunks && indptr_out && nnz_out, "sg_chunks_to_csr: null pointer argument");
  SG_ARG(n_rows >= 0 && chunk_rows >= 1 && chunk_cols >= 1 && n_rows <= chunk_rows && n_cols >= 1 &&
             n_cols < (int64_t(1) << 31) && indptr_base >= 0 && capacity >= 0,
         "sg_chunks_to_csr: bad sizes");
  SG_ARG(capacity == 0 || (indices_out && data_out), "sg_chunks_to_csr: null output arrays");
  const bool count_only = capacity == 0;
  if (n_rows == 0) {
    SG_CUDA(cudaMemcpyAsync(indptr_out, &indptr_base, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    SG_CUDA(cudaStreamSynchronize(st));
    *nnz_out = 0;
    return SG_OK;
  }
  const size_t need = sg::Carver::need(sizeof(int64_t) * size_t(n_rows)) + sg::Carver::need(sizeof(int));
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  int64_t* cnt = cv.take<int64_t>(size_t(n_rows));
  int* err = cv.take<int>(1);
  SG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  const unsigned grid = unsigned(sg::ceil_div(n_rows * 32, 256));
  chunk_row_count_kernel<<<grid, 256, 0, st>>>(chunks, n_rows, chunk_rows, chunk_cols, n_cols, cnt, err);
  SG_LAUNCH_CHECK();
  row_scan_kernel<<<1, 1024, 0, st>>>(cnt, n_rows, indptr_base, indptr_out);
  SG_LAUNCH_CHECK();
  if (!count_only) {
    chunk_row_scatter_kernel<<<grid, 256, 0, st>>>(chunks, n_rows, chunk_rows, chunk_cols, n_cols, indptr_out,
                                                   indptr_base, capacity, indices_out, data_out);
    SG_LAUNCH_CHECK();
  }
  int64_t last = 0;
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&last, indptr_out + n_rows, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  *nnz_out = last - indptr_base;
  if (herr) return sg::fail(SG_ERR_ARG, "sg_chunks_to_csr: a count above 2^31 - 1 does not fit int32 CSR data");
  if (!count_only && *nnz_out > capacity)
    return sg::fail(SG_ERR_ARG, "sg_chunks_to_csr: %lld non-zeros, more than the capacity of %lld",
                    (long long)*nnz_out, (long long)capacity);
  return SG_OK;
}
