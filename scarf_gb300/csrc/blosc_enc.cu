// f2, writing: Blosc1 frames of device bytes, the chunk format scarf's stores
// are written in (create_zarr_dataset, scarf/writers.py:58-89: numcodecs
// Blosc, LZ4 codec, bit shuffle). The formats are those the decoder in
// blosc.cu reads:
//
// * frame: 16-byte header (version 2, LZ4 format version 1, flags, type size;
//   uncompressed bytes, block size, frame bytes, little-endian), one int32
//   start offset per block, then per block an int32 size and the LZ4 stream,
//   or the block's bytes as they are when that size equals the block length.
//   Flags written: 0x04 bit shuffle or 0x01 byte shuffle, 0x10 (blocks not
//   split into per-byte streams), codec 1 (LZ4) in bits 5-7.
// * bit shuffle of a block of n elements of ts bytes: for n rounded down to
//   a multiple of 8, bit j of byte b of element e goes to bit e (LSB first)
//   of bit-plane 8 b + j; the remaining elements and bytes are stored as they
//   are. Byte shuffle stores byte b of every element together.
// * LZ4 block: greedy matches of at least 4 bytes found through a hash table
//   of 4-byte prefixes; every sequence is a token, the literal-length bytes,
//   the literals, a 16-bit offset and the match-length bytes; the last
//   sequence is literals only. As the format requires, no match starts in the
//   last 12 bytes and the last 5 bytes are literals.
//
// shuffle_bit_kernel: a warp per 32 elements of a block; lane i holds 4 bytes
// of element i, and one ballot per bit-plane gathers the plane's 32 bits.
// lz4_encode_kernel: a thread per block (blocks are at most 32 KB), its hash
// table of 2^10 positions in shared memory; every write is checked against
// the block's length, and a block whose stream would not be shorter is
// stored as it is. pack_kernel: a warp per block copies the size word and the
// stream to the block's place in the frames.
#include "common.cuh"

#include <cstring>
#include <vector>

namespace {

constexpr int kEncMaxBlock = 32768;   // table entries hold position + 1 in 16 bits
constexpr int kHashBits = 10;
constexpr int kEncThreads = 32;       // blocks per CTA

struct EncBlock {
  int64_t off;      // offset of the block in the source (and in the staging and compressed buffers)
  int64_t dst;      // offset of the block's size word in the frames (set after compression)
  int32_t len;
  int32_t typesize;
};

__global__ void shuffle_bit_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ stage,
                                   const EncBlock* __restrict__ blocks, const int64_t* __restrict__ group_start,
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
  const EncBlock b = blocks[lo];
  const int ts = b.typesize;
  const int64_t n = b.len / ts;
  const int64_t n8 = n - n % 8;
  const int64_t plane_bytes = n8 / 8;
  const int64_t e0 = (gw - group_start[lo]) * 32;
  const uint8_t* in = src + b.off;
  uint8_t* o = stage + b.off;
  // elements past the last multiple of 8, and bytes past the last whole element, stay as they are
  for (int64_t i = max(e0, n8) * ts + lane; i < min(n, e0 + 32) * ts; i += 32) o[i] = in[i];
  if (e0 + 32 >= n)
    for (int64_t i = n * ts + lane; i < b.len; i += 32) o[i] = in[i];
  if (e0 >= n8) return;
  const int cnt = int(n8 - e0 < 32 ? n8 - e0 : 32);  // a multiple of 8
  for (int g = 0; g < (ts + 3) / 4; ++g) {
    // lane i: bytes 4g .. 4g+3 of element e0 + i
    uint32_t word = 0;
    if (lane < cnt) {
      const uint8_t* el = in + (e0 + lane) * ts;
      for (int q = 0; q < 4 && 4 * g + q < ts; ++q) word |= uint32_t(el[4 * g + q]) << (8 * q);
    }
    uint32_t mine = 0;
    for (int q = 0; q < 32; ++q) {
      const uint32_t m = __ballot_sync(0xffffffffu, (word >> q) & 1u);
      if (lane == q) mine = m;
    }
    const int p = 32 * g + lane;  // this lane's bit-plane
    if (p < 8 * ts) {
      uint8_t* pl = o + int64_t(p) * plane_bytes + e0 / 8;
      for (int q = 0; q < cnt / 8; ++q) pl[q] = uint8_t(mine >> (8 * q));
    }
  }
}

// a CTA per block
__global__ void shuffle_byte_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ stage,
                                    const EncBlock* __restrict__ blocks) {
  const EncBlock b = blocks[blockIdx.x];
  const int ts = b.typesize;
  const int64_t n = b.len / ts;
  const uint8_t* in = src + b.off;
  uint8_t* o = stage + b.off;
  for (int64_t i = threadIdx.x; i < b.len; i += blockDim.x) {
    if (i < n * ts) {
      const int64_t e = i / ts;
      const int bb = int(i - e * ts);
      o[int64_t(bb) * n + e] = in[i];
    } else {
      o[i] = in[i];
    }
  }
}

__device__ __forceinline__ uint32_t ld32(const uint8_t* p) {
  return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}

// One LZ4 sequence: `lit` literals from s + anchor, then (unless last) a match
// of `ml` bytes at distance `off`. False when it would not fit in `cap` bytes.
__device__ bool lz4_emit(const uint8_t* s, int anchor, int lit, int off, int ml, bool last, uint8_t* o, int& op,
                         int cap) {
  const int need = 1 + lit + (lit >= 15 ? (lit - 15) / 255 + 1 : 0) +
                   (last ? 0 : 2 + (ml - 4 >= 15 ? (ml - 4 - 15) / 255 + 1 : 0));
  if (op + need > cap) return false;
  o[op++] = uint8_t(((lit < 15 ? lit : 15) << 4) | (last ? 0 : (ml - 4 < 15 ? ml - 4 : 15)));
  if (lit >= 15) {
    int v = lit - 15;
    for (; v >= 255; v -= 255) o[op++] = 255;
    o[op++] = uint8_t(v);
  }
  for (int i = 0; i < lit; ++i) o[op++] = s[anchor + i];
  if (!last) {
    o[op++] = uint8_t(off & 255);
    o[op++] = uint8_t(off >> 8);
    if (ml - 4 >= 15) {
      int v = ml - 4 - 15;
      for (; v >= 255; v -= 255) o[op++] = 255;
      o[op++] = uint8_t(v);
    }
  }
  return true;
}

__global__ void __launch_bounds__(kEncThreads)
lz4_encode_kernel(const uint8_t* __restrict__ stage, uint8_t* __restrict__ comp, const EncBlock* __restrict__ blocks,
                  int n_blocks, int32_t* __restrict__ csize) {
  extern __shared__ uint16_t enc_tab[];
  const int bi = blockIdx.x * kEncThreads + threadIdx.x;
  if (bi >= n_blocks) return;
  uint16_t* tab = enc_tab + threadIdx.x * (1 << kHashBits);
  for (int i = 0; i < (1 << kHashBits); ++i) tab[i] = 0;
  const EncBlock b = blocks[bi];
  const uint8_t* s = stage + b.off;
  uint8_t* o = comp + b.off;
  const int n = b.len;
  const int cap = n - 1;  // a stream of n bytes or more is stored as the block itself
  int op = 0, anchor = 0, ip = 0;
  bool ok = cap > 0;
  if (ok && n >= 13) {
    const int mflimit = n - 12;    // no match starts in the last 12 bytes
    const int matchlimit = n - 5;  // the last 5 bytes are literals
    while (ip < mflimit) {
      const uint32_t seq = ld32(s + ip);
      const uint32_t hh = (seq * 2654435761u) >> (32 - kHashBits);
      const int ref = int(tab[hh]) - 1;
      tab[hh] = uint16_t(ip + 1);
      if (ref >= 0 && ld32(s + ref) == seq) {
        int ml = 4;
        while (ip + ml < matchlimit && s[ref + ml] == s[ip + ml]) ++ml;
        if (!lz4_emit(s, anchor, ip - anchor, ip - ref, ml, false, o, op, cap)) {
          ok = false;
          break;
        }
        ip += ml;
        anchor = ip;
      } else {
        ip += 1 + ((ip - anchor) >> 6);  // step faster through stretches without matches
      }
    }
  }
  if (ok) ok = lz4_emit(s, anchor, n - anchor, 0, 0, true, o, op, cap);
  csize[bi] = ok ? op : n;
}

// a warp per block: the size word, then the stream (or the block as it is)
__global__ void pack_kernel(const uint8_t* __restrict__ stage, const uint8_t* __restrict__ comp,
                            const EncBlock* __restrict__ blocks, const int32_t* __restrict__ csize, int n_blocks,
                            uint8_t* __restrict__ frames) {
  const int lane = threadIdx.x & 31;
  const int64_t bi = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (bi >= n_blocks) return;
  const EncBlock b = blocks[bi];
  const int32_t cs = csize[bi];
  uint8_t* o = frames + b.dst;
  if (lane < 4) o[lane] = uint8_t(uint32_t(cs) >> (8 * lane));
  const uint8_t* in = (cs == b.len ? stage : comp) + b.off;
  for (int i = lane; i < cs; i += 32) o[4 + i] = in[i];
}

void put32(uint8_t* p, uint32_t v) {
  for (int q = 0; q < 4; ++q) p[q] = uint8_t(v >> (8 * q));
}

int64_t frame_bound(int64_t len, int64_t bs) {
  const int64_t nb = len == 0 ? 0 : (len + bs - 1) / bs;
  return 16 + 4 * nb + 4 * nb + len;
}

}  // namespace

extern "C" int64_t sg_blosc_encode_bound(const int64_t* chunk_offsets, int32_t n_chunks, int32_t blocksize) {
  if (!chunk_offsets || n_chunks < 0 || blocksize <= 0) return -1;
  int64_t t = 0;
  for (int c = 0; c < n_chunks; ++c) t += frame_bound(chunk_offsets[c + 1] - chunk_offsets[c], blocksize);
  return t;
}

extern "C" int sg_blosc_encode(sg_handle* h, const void* src, const int64_t* chunk_offsets, int32_t n_chunks,
                               int32_t typesize, int32_t shuffle, int32_t blocksize, void* frames_out,
                               int64_t frames_capacity, int64_t* frame_offsets_out, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(n_chunks >= 0 && (n_chunks == 0 || (src && chunk_offsets && frames_out && frame_offsets_out)),
         "sg_blosc_encode: null pointer argument");
  SG_ARG(typesize >= 1 && typesize <= 255, "sg_blosc_encode: type size %d outside 1..255", typesize);
  SG_ARG(shuffle >= 0 && shuffle <= 2, "sg_blosc_encode: shuffle must be 0 (none), 1 (byte) or 2 (bit)");
  SG_ARG(blocksize >= typesize && blocksize <= kEncMaxBlock && blocksize % typesize == 0,
         "sg_blosc_encode: block size %d must be a multiple of the type size, at most %d", blocksize, kEncMaxBlock);
  if (n_chunks == 0) {
    if (frame_offsets_out) frame_offsets_out[0] = 0;
    return SG_OK;
  }
  const int64_t base = chunk_offsets[0];
  for (int c = 0; c < n_chunks; ++c) {
    const int64_t len = chunk_offsets[c + 1] - chunk_offsets[c];
    SG_ARG(len >= 0 && len < (int64_t(1) << 31) - 64, "sg_blosc_encode: chunk %d has %lld bytes", c, (long long)len);
  }
  const int64_t bound = sg_blosc_encode_bound(chunk_offsets, n_chunks, blocksize);
  SG_ARG(frames_capacity >= bound, "sg_blosc_encode: %lld bytes of frames capacity, %lld needed",
         (long long)frames_capacity, (long long)bound);
  // blocks of every chunk; a chunk shorter than the block size is one block
  std::vector<EncBlock> blocks;
  std::vector<int> first(n_chunks + 1, 0);
  std::vector<int64_t> group_start;
  int64_t groups = 0;
  for (int c = 0; c < n_chunks; ++c) {
    first[c] = int(blocks.size());
    const int64_t off = chunk_offsets[c] - base;
    const int64_t len = chunk_offsets[c + 1] - chunk_offsets[c];
    for (int64_t a = 0; a < len; a += blocksize) {
      const int32_t bl = int32_t(std::min<int64_t>(blocksize, len - a));
      blocks.push_back({off + a, 0, bl, typesize});
      group_start.push_back(groups);
      groups += std::max<int64_t>(1, ((bl / typesize) + 31) / 32);
    }
  }
  first[n_chunks] = int(blocks.size());
  const int nb = int(blocks.size());
  const int64_t total = chunk_offsets[n_chunks] - base;
  // a one-byte type is stored unshuffled (no shuffle flag)
  const int shuf = typesize > 1 ? shuffle : 0;
  const bool shuffled = shuf != 0;
  const size_t need = (shuffled ? sg::Carver::need(size_t(total)) : 0) + sg::Carver::need(size_t(total) + 1) +
                      sg::Carver::need(sizeof(EncBlock) * size_t(nb) + 8) +
                      sg::Carver::need(sizeof(int64_t) * size_t(nb) + 8) +
                      sg::Carver::need(sizeof(int32_t) * size_t(nb) + 8) + sg::Carver::need(size_t(bound));
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  uint8_t* d_stage = shuffled ? cv.take<uint8_t>(size_t(total)) : nullptr;
  uint8_t* d_comp = cv.take<uint8_t>(size_t(total) + 1);
  EncBlock* d_blocks = cv.take<EncBlock>(size_t(nb) + 1);
  int64_t* d_gs = cv.take<int64_t>(size_t(nb) + 1);
  int32_t* d_cs = cv.take<int32_t>(size_t(nb) + 1);
  uint8_t* d_frames = cv.take<uint8_t>(size_t(bound));
  const uint8_t* d_src = static_cast<const uint8_t*>(src) + base;
  const uint8_t* d_in = shuffled ? d_stage : d_src;
  sg::ProfScope prof(h, "blosc_encode", st);
  if (nb > 0) {
    SG_CUDA(cudaMemcpyAsync(d_blocks, blocks.data(), sizeof(EncBlock) * size_t(nb), cudaMemcpyHostToDevice, st));
    if (shuf == 2) {
      SG_CUDA(cudaMemcpyAsync(d_gs, group_start.data(), sizeof(int64_t) * size_t(nb), cudaMemcpyHostToDevice, st));
      shuffle_bit_kernel<<<unsigned(sg::ceil_div(groups * 32, 256)), 256, 0, st>>>(d_src, d_stage, d_blocks, d_gs,
                                                                                     nb, groups);
      SG_LAUNCH_CHECK();
    } else if (shuf == 1) {
      shuffle_byte_kernel<<<unsigned(nb), 256, 0, st>>>(d_src, d_stage, d_blocks);
      SG_LAUNCH_CHECK();
    }
    const size_t tab_bytes = sizeof(uint16_t) * kEncThreads * (1u << kHashBits);
    SG_CUDA(cudaFuncSetAttribute(lz4_encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tab_bytes)));
    lz4_encode_kernel<<<unsigned(sg::ceil_div_i(nb, kEncThreads)), kEncThreads, tab_bytes, st>>>(d_in, d_comp,
                                                                                                  d_blocks, nb, d_cs);
    SG_LAUNCH_CHECK();
  }
  std::vector<int32_t> cs(size_t(nb) + 1, 0);
  if (nb > 0) {
    SG_CUDA(cudaMemcpyAsync(cs.data(), d_cs, sizeof(int32_t) * size_t(nb), cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
  }
  // frame layout: header, block starts, then each block's size word and stream
  std::vector<int64_t> fo(size_t(n_chunks) + 1, 0);
  for (int c = 0; c < n_chunks; ++c) {
    int64_t pos = 16 + 4 * int64_t(first[c + 1] - first[c]);
    for (int b = first[c]; b < first[c + 1]; ++b) {
      blocks[b].dst = fo[c] + pos;
      pos += 4 + cs[b];
    }
    fo[c + 1] = fo[c] + pos;
  }
  if (nb > 0) {
    SG_CUDA(cudaMemcpyAsync(d_blocks, blocks.data(), sizeof(EncBlock) * size_t(nb), cudaMemcpyHostToDevice, st));
    pack_kernel<<<unsigned(sg::ceil_div(int64_t(nb) * 32, 256)), 256, 0, st>>>(d_in, d_comp, d_blocks, d_cs, nb,
                                                                               d_frames);
    SG_LAUNCH_CHECK();
  }
  uint8_t* out = static_cast<uint8_t*>(frames_out);
  if (fo[n_chunks] > 0)
    SG_CUDA(cudaMemcpyAsync(out, d_frames, size_t(fo[n_chunks]), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  const uint8_t flags = uint8_t((1 << 5) | 0x10 | (shuf == 2 ? 0x04 : shuf == 1 ? 0x01 : 0));
  for (int c = 0; c < n_chunks; ++c) {
    uint8_t* f = out + fo[c];
    const int64_t len = chunk_offsets[c + 1] - chunk_offsets[c];
    f[0] = 2;  // Blosc1 format version
    f[1] = 1;  // LZ4 format version
    f[2] = flags;
    f[3] = uint8_t(typesize);
    put32(f + 4, uint32_t(len));
    put32(f + 8, uint32_t(std::min<int64_t>(blocksize, len)));
    put32(f + 12, uint32_t(fo[c + 1] - fo[c]));
    for (int b = first[c]; b < first[c + 1]; ++b) put32(f + 16 + 4 * (b - first[c]), uint32_t(blocks[b].dst - fo[c]));
  }
  for (int c = 0; c <= n_chunks; ++c) frame_offsets_out[c] = fo[c];
  return SG_OK;
}
