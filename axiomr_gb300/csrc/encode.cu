// Output encoding: framebuffers as PNG files, built on the GPU.
//
// The reference shows a frame by copying the BGRA8 colour plane into a bottom-up 32-bit
// DIB and blitting it to a window (Window::present, src/window.cpp:70-84; the DIB header,
// src/windows_bitmap.cpp:15-30): the alpha byte is not shown and framebuffer row 0 is the
// bottom row of the picture. The headless counterpart here is one PNG file per framebuffer,
// top row first, RGB8 (what the window shows) or RGBA8.
//
// File layout (PNG: ISO/IEC 15948; zlib: RFC 1950; deflate: RFC 1951):
//   signature, IHDR, a tEXt chunk ("Software") whose length puts the first IDAT data byte
//   at file offset 80, IDAT chunks of kIdat data bytes each (the last one shorter), IEND.
//   From one IDAT chunk's data to the next is kChunkStride = 65536 bytes, so every 32-bit
//   word of the compressed stream lies at a 4-byte aligned file offset inside one chunk.
//   The IDAT data is one zlib stream: header 78 01, one deflate block with the fixed
//   Huffman codes, Adler-32. Every scanline has filter type 0 (None).
// Compression: per scanline, runs of pixels equal to their left neighbour become matches
//   at distance 3 / 4 bytes, runs of pixels equal to the ones above matches at one scanline,
//   everything else literals. Runs are cut every 32 pixels (one warp step), so that a warp
//   finds them with ballots and every step's bits are known without a sequential parse;
//   a flat 32-pixel step costs 12-13 bits.
//
// Four launches per call, each over all images of the call:
//   rows   : one warp per scanline, 32 pixels per step: runs, bit counts (warp scan), the
//            codes assembled in shared memory and written as whole words to the scanline's
//            slot in a staging buffer; the Adler-32 partial sums of the scanline
//   layout : one block per image; exclusive scan of the scanline bit counts, then
//            signature, IHDR, tEXt, the IDAT chunk headers, IEND, the Adler-32, file size
//   pack   : one block per 8 scanlines of an image, one thread per 32-bit word of the
//            compressed stream: gathers its bits from the staged scanlines (zlib and block
//            headers, end-of-block, Adler-32 included) and stores the word; no word is
//            written twice, so no atomics
//   crc    : one block per IDAT chunk: CRC-32 of its type and data
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "api_internal.h"
#include "api_types.h"

using namespace axr_internal;

namespace axr {

constexpr uint32_t kIdat = 65524;         // data bytes of a full IDAT chunk (multiple of 4)
constexpr uint32_t kChunkStride = 65536;  // kIdat + 12: chunk length, type and CRC
constexpr uint32_t kData0 = 80;           // file offset of the first IDAT data byte
constexpr uint32_t kHeaderBits = 19;      // zlib header (16 bits) + deflate block header (3)
constexpr uint32_t kCrcPoly = 0xEDB88320u;  // CRC-32 polynomial, bit-reflected
constexpr uint32_t kAdlerMod = 65521u;
constexpr int kPngWarps = 8;
constexpr int kLayoutThreads = 1024;

struct PngJob {
    const uint32_t* color;          // BGRA8 plane, row 0 = bottom
    uint8_t* out;                   // file buffer (device)
    unsigned long long* size;       // file size out (device); 0 when the image did not fit
    unsigned long long capacity;
    unsigned long long stage_base;  // first staging word of this image's scanline slots
    uint32_t width, height, channels, row_bytes;
    uint32_t row_words;   // staging words per scanline slot
    uint32_t row_base;    // first scanline of this image in the call's scanline arrays
    uint32_t max_chunks;  // IDAT chunks of the worst case
    unsigned long long max_words;  // stream words of the worst case
};

struct PngLayout {
    unsigned long long end_bit;       // end of the last scanline's bits in the stream
    unsigned long long stream_bytes;  // zlib stream length (IDAT data bytes in all)
    uint32_t chunks;                  // IDAT chunks
    uint32_t adler;                   // Adler-32 of the scanline bytes
    uint32_t error;                   // the file would exceed the buffer
    uint32_t pad;
};

struct PngParams {
    const PngJob* jobs;
    PngLayout* layout;
    uint32_t* stage;           // scanline slots
    uint32_t* row_bits;        // per scanline: its bits (filter byte included)
    uint32_t* s0;              // per scanline: sum of its bytes
    unsigned long long* s1;    // per scanline: sum of (row_bytes - i) * byte_i
    unsigned long long* row_off;  // per scanline: first bit in the stream
    const uint2* groups;       // pack blocks: (image, first scanline) of 32-scanline groups
    uint32_t jobs_n, rows;
    uint32_t crc_table[256];   // byte-at-a-time table of the reflected polynomial
    uint32_t xpow[32];         // x^(2^k) mod P, bit-reflected
    // full IDAT chunks (type + 65524 data bytes): x^(8 a_t) for the bytes a_t after thread
    // t's 256-byte part, and 0xFFFFFFFF * x^(8 * 65528) (the initial value's term)
    uint32_t full_shift[256];
    uint32_t full_init;
};

constexpr uint32_t kGroupRows = 8;  // scanlines per pack block

constexpr int kBufWords = 40;  // shared words per warp: one 32-pixel step (<= 1152 bits) + carry
constexpr uint32_t kCrcJobs = 1024;  // images whose chunk offsets a crc block keeps in shared memory

// ------------------------------------------------------------------ device helpers

__device__ __forceinline__ uint32_t find_job(const PngJob* jobs, uint32_t n, uint32_t row) {
    uint32_t lo = 0, hi = n;  // the last job with row_base <= row
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&jobs[mid].row_base) <= row) lo = mid; else hi = mid;
    }
    return lo;
}

// file offset of byte b of the zlib stream
__device__ __forceinline__ size_t stream_offset(unsigned long long b) {
    return kData0 + (size_t)(b / kIdat) * kChunkStride + (size_t)(b % kIdat);
}

__device__ __forceinline__ uint32_t reverse_bits(uint32_t code, uint32_t len) { return __brev(code) >> (32 - len); }

// deflate length symbol (257..285), its extra bits and their value, for 3 <= len <= 258
__device__ __forceinline__ void length_symbol(uint32_t len, uint32_t& sym, uint32_t& ebits, uint32_t& extra) {
    if (len == 258) {
        sym = 285; ebits = 0; extra = 0;
        return;
    }
    const uint32_t v = len - 3;
    if (v < 8) {
        sym = 257 + v; ebits = 0; extra = 0;
        return;
    }
    const uint32_t e = (31 - __clz(v)) - 2, m = (v >> e) & 3u;
    sym = 257 + 4 * (e + 1) + m;
    ebits = e;
    extra = v - ((4 + m) << e);
}

// deflate distance code (0..29), its extra bits and their value, for 1 <= dist <= 32768
__device__ __forceinline__ void distance_code(uint32_t dist, uint32_t& code, uint32_t& ebits, uint32_t& extra) {
    const uint32_t v = dist - 1;
    if (v < 4) {
        code = v; ebits = 0; extra = 0;
        return;
    }
    const uint32_t e = (31 - __clz(v)) - 1, m = (v >> e) & 1u;
    code = 2 * (e + 1) + m;
    ebits = e;
    extra = v - ((2 + m) << e);
}

// fixed Huffman code of a literal/length symbol: (code bits already reversed, length)
__device__ __forceinline__ void litlen_code(uint32_t sym, uint32_t& bits, uint32_t& len) {
    if (sym < 144) { bits = reverse_bits(0x30 + sym, 8); len = 8; }
    else if (sym < 256) { bits = reverse_bits(0x190 + (sym - 144), 9); len = 9; }
    else if (sym < 280) { bits = reverse_bits(sym - 256, 7); len = 7; }
    else { bits = reverse_bits(0xC0 + (sym - 280), 8); len = 8; }
}

__device__ __forceinline__ uint32_t literal_bits(uint32_t byte) { return byte < 144 ? 8u : 9u; }

// fixed Huffman code of literal byte b, reversed for the LSB-first stream; returns its length
__device__ __forceinline__ uint32_t literal_code(uint32_t b, uint32_t& code) {
    const bool hi = b >= 144;
    code = hi ? (__brev(0x190u + b - 144u) >> 23) : (__brev(0x30u + b) >> 24);
    return hi ? 9u : 8u;
}

__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// ------------------------------------------------------------------ kernels

// A warp's code buffer: buf[0] holds staging word wbase of its scanline. After codes up
// to bit `end` are in, whole words go out to the staging slot and the partial one moves
// to buf[0]. Warp-uniform.
__device__ __forceinline__ void flush_words(uint32_t* buf, uint32_t* stage, uint32_t row_words, uint32_t& wbase,
                                            uint32_t& nbits, uint32_t end, int lane) {
    const uint32_t done = (end >> 5) - wbase;
    if (done) {
        for (uint32_t k = (uint32_t)lane; k < done; k += 32)
            if (wbase + k < row_words) stage[wbase + k] = buf[k];  // the slot holds the worst case
        const uint32_t carry = buf[done];
        __syncwarp();
        for (uint32_t k = (uint32_t)lane; k <= done; k += 32) buf[k] = 0u;
        __syncwarp();
        if (lane == 0) buf[0] = carry;
        __syncwarp();
        wbase += done;
    }
    nbits = end;
}

// One code of n <= 31 bits appended by lane 0 (warp-uniform).
__device__ __forceinline__ void put_uniform(uint32_t* buf, uint32_t* stage, uint32_t row_words, uint32_t& wbase,
                                            uint32_t& nbits, unsigned long long code, uint32_t n, int lane) {
    if (lane == 0) {
        const uint32_t pos = nbits - wbase * 32, k = pos >> 5, sh = pos & 31u;
        const unsigned long long lo = code << sh;
        buf[k] |= (uint32_t)lo;
        buf[k + 1] |= (uint32_t)(lo >> 32);
    }
    __syncwarp();
    flush_words(buf, stage, row_words, wbase, nbits, nbits + n, lane);
}

// the code of one match of `len` bytes at distance code (dc, deb, dex)
__device__ __forceinline__ uint32_t match_code(uint32_t len, uint32_t dc, uint32_t deb, uint32_t dex,
                                               unsigned long long& code) {
    uint32_t sym, eb, ex, bits, n;
    length_symbol(len, sym, eb, ex);
    litlen_code(sym, bits, n);
    code = bits;
    code |= (unsigned long long)ex << n;
    n += eb;
    code |= (unsigned long long)reverse_bits(dc, 5) << n;
    n += 5;
    code |= (unsigned long long)dex << n;
    return n + deb;
}

// One warp per scanline. Per 32-pixel step, lane i takes pixel x = step + i: it is in a
// left run when it equals pixel x-1, else in an up run when it equals the pixel above; a
// run starts where its kind starts in the step and ends where it ends or at the step's end.
// A run start emits one match of the run's length, a lone up-run pixel whose match would
// cost at least its literals emits literals instead, other pixels emit literals. Steps that
// lie wholly in a left run (flat regions) are merged into matches of up to 258 bytes; a step
// wholly equal to the scanline above is one match.
template <int C>
__global__ void __launch_bounds__(32 * kPngWarps, 6) png_rows_kernel(const __grid_constant__ PngParams p) {
    __shared__ uint32_t s_buf[kPngWarps][kBufWords];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t row = blockIdx.x * kPngWarps + (uint32_t)warp;
    if (row >= p.rows) return;
    const PngJob& j = p.jobs[find_job(p.jobs, p.jobs_n, row)];
    const uint32_t W = j.width, H = j.height, L = j.row_bytes, row_words = j.row_words;
    const uint32_t r = row - j.row_base;
    const uint32_t mask = C == 4 ? 0xFFFFFFFFu : 0x00FFFFFFu;
    const uint32_t* src = j.color + (size_t)(H - 1 - r) * W;
    const bool has_up = r > 0 && L <= 32768u;
    const uint32_t* up = src + W;  // the framebuffer row above = the previous scanline
    uint32_t* stage = p.stage + j.stage_base + (size_t)r * row_words;
    uint32_t up_code, up_eb, up_ex;
    distance_code(has_up ? L : 1u, up_code, up_eb, up_ex);
    uint32_t left_code, left_eb, left_ex;
    distance_code(C, left_code, left_eb, left_ex);
    constexpr uint32_t kMaxRun = 258u / C;  // pixels in the longest match
    unsigned long long full_code, up32_code;
    const uint32_t full_bits = match_code(kMaxRun * C, left_code, left_eb, left_ex, full_code);
    const uint32_t up32_bits = match_code(32 * C, up_code, up_eb, up_ex, up32_code);

    uint32_t* buf = s_buf[warp];
    for (int k = lane; k < kBufWords; k += 32) buf[k] = 0u;
    __syncwarp();
    if (lane == 0) buf[0] = reverse_bits(0x30, 8);  // filter type 0 as a literal byte
    uint32_t nbits = 8;    // bits of this scanline so far
    uint32_t wbase = 0;    // staging word that buf[0] holds
    uint32_t prev = 0;     // the pixel before this step
    uint32_t pending = 0;  // pixels of a left run carried over whole steps, not yet emitted
    uint32_t a0 = 0;                    // Adler-32 partial sums of this lane's bytes
    unsigned long long a1 = 0;
    __syncwarp();
    for (uint32_t c0 = 0; c0 < W; c0 += 32) {
        const uint32_t x = c0 + (uint32_t)lane;
        const bool valid = x < W;
        const uint32_t raw = valid ? __ldg(src + x) : 0u;
        const uint32_t v = raw & mask;
        // Adler-32 partial sums: byte i of the scanline (i = 0 is the filter byte, 0) adds
        // (L - i) * byte: (L - i) * (b0 + b1 + b2 [+ b3]) - (b1 + 2 b2 [+ 3 b3]) per pixel
        if (valid) {
            const uint32_t b1 = (raw >> 8) & 255u, b2 = raw & 255u;
            uint32_t sum = ((raw >> 16) & 255u) + b1 + b2, lag = b1 + 2 * b2;
            if (C == 4) {
                sum += raw >> 24;
                lag += 3 * (raw >> 24);
            }
            a0 += sum;
            a1 += (unsigned long long)(L - 1 - x * C) * sum - lag;
        }
        uint32_t left = __shfl_up_sync(0xFFFFFFFFu, v, 1);
        if (lane == 0) left = prev;
        const bool eq_l = valid && x > 0 && v == left;
        const unsigned m_l = __ballot_sync(0xFFFFFFFFu, eq_l);
        if (m_l == 0xFFFFFFFFu) {  // the whole step continues a left run
            pending += 32;
            if (pending >= kMaxRun) {
                put_uniform(buf, stage, row_words, wbase, nbits, full_code, full_bits, lane);
                pending -= kMaxRun;
            }
            continue;  // prev is unchanged: every pixel equals it
        }
        if (pending) {
            unsigned long long c;
            const uint32_t n = match_code(pending * C, left_code, left_eb, left_ex, c);
            put_uniform(buf, stage, row_words, wbase, nbits, c, n, lane);
            pending = 0;
        }
        const uint32_t u = (valid && has_up) ? (__ldg(up + x) & mask) : 0u;
        const bool eq_u = valid && has_up && !eq_l && v == u;
        const unsigned m_u = __ballot_sync(0xFFFFFFFFu, eq_u);
        prev = __shfl_sync(0xFFFFFFFFu, v, 31);
        if (m_u == 0xFFFFFFFFu) {  // the whole step repeats the scanline above
            put_uniform(buf, stage, row_words, wbase, nbits, up32_code, up32_bits, lane);
            continue;
        }
        const unsigned m = eq_l ? m_l : m_u;
        const bool start = (eq_l || eq_u) && !((m << 1) >> lane & 1u);
        const uint32_t run = start ? (uint32_t)__ffsll(~((unsigned long long)m >> lane)) - 1u : 0u;
        uint32_t lit_bits = 0;
        if (valid) {
            lit_bits = (((v >> 16) & 255u) < 144 ? 8u : 9u) + (((v >> 8) & 255u) < 144 ? 8u : 9u) +
                       ((v & 255u) < 144 ? 8u : 9u);
            if (C == 4) lit_bits += (v >> 24) < 144 ? 8u : 9u;
        }
        const bool lone_up = eq_u && start && run == 1 && 12u + up_eb >= lit_bits;
        const bool literal = valid && (!(eq_l || eq_u) || lone_up);
        const bool match = start && !lone_up;
        unsigned long long code = 0;
        uint32_t n = 0;
        if (literal) {
            uint32_t c, k;
            k = literal_code((v >> 16) & 255u, c); code = c; n = k;
            k = literal_code((v >> 8) & 255u, c);  code |= (unsigned long long)c << n; n += k;
            k = literal_code(v & 255u, c);         code |= (unsigned long long)c << n; n += k;
            if (C == 4) { k = literal_code(v >> 24, c); code |= (unsigned long long)c << n; n += k; }
        } else if (match) {
            n = eq_l ? match_code(run * C, left_code, left_eb, left_ex, code)
                     : match_code(run * C, up_code, up_eb, up_ex, code);
        }
        // bit position of this lane's codes
        uint32_t incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += t;
        }
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        if (n) {
            const uint32_t pos = nbits + incl - n - wbase * 32;  // bit within buf
            const uint32_t k = pos >> 5, sh = pos & 31u;
            const unsigned long long lo = code << sh;
            const uint32_t w0 = (uint32_t)lo, w1 = (uint32_t)(lo >> 32), w2 = sh ? (uint32_t)(code >> (64 - sh)) : 0u;
            if (w0) atomicOr(&buf[k], w0);
            if (w1) atomicOr(&buf[k + 1], w1);
            if (w2) atomicOr(&buf[k + 2], w2);
        }
        __syncwarp();
        flush_words(buf, stage, row_words, wbase, nbits, nbits + total, lane);
    }
    if (pending) {
        unsigned long long c;
        const uint32_t n = match_code(pending * C, left_code, left_eb, left_ex, c);
        put_uniform(buf, stage, row_words, wbase, nbits, c, n, lane);
    }
    if (lane == 0 && (nbits & 31u) && wbase < row_words) stage[wbase] = buf[0];
    const unsigned long long s0 = warp_sum64(a0);
    a1 = warp_sum64(a1);
    if (lane == 0) {
        p.row_bits[row] = nbits;
        p.s0[row] = (uint32_t)s0;
        p.s1[row] = a1;
    }
}

__device__ __forceinline__ uint32_t crc_bytes(const uint32_t* table, uint32_t crc, const uint8_t* b, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) crc = table[(crc ^ b[i]) & 255u] ^ (crc >> 8);
    return crc;
}

__device__ __forceinline__ void put_be32(uint8_t* p, uint32_t v) {
    p[0] = (uint8_t)(v >> 24);
    p[1] = (uint8_t)(v >> 16);
    p[2] = (uint8_t)(v >> 8);
    p[3] = (uint8_t)v;
}

// a chunk's CRC over its type and data (at p[4..8+n)), written after the data
__device__ void seal_chunk(const uint32_t* table, uint8_t* p, uint32_t n) {
    const uint32_t crc = crc_bytes(table, 0xFFFFFFFFu, p + 4, 4 + n) ^ 0xFFFFFFFFu;
    put_be32(p + 8 + n, crc);
}

__global__ void __launch_bounds__(kLayoutThreads) png_layout_kernel(const __grid_constant__ PngParams p) {
    __shared__ uint32_t s_table[256];
    __shared__ unsigned long long s_warp[kLayoutThreads / 32];
    __shared__ unsigned long long s_a[kLayoutThreads / 32], s_b[kLayoutThreads / 32];
    __shared__ unsigned long long s_carry;
    const PngJob& j = p.jobs[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < 256; k += kLayoutThreads) s_table[k] = p.crc_table[k];
    if (tid == 0) s_carry = kHeaderBits;
    __syncthreads();
    // exclusive scan of the scanline bit counts
    for (uint32_t c0 = 0; c0 < j.height; c0 += kLayoutThreads) {
        const uint32_t r = c0 + (uint32_t)tid;
        const unsigned long long v = r < j.height ? p.row_bits[j.row_base + r] : 0ull;
        unsigned long long incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w += t;
            }
            s_warp[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const unsigned long long base = s_carry + (warp ? s_warp[warp - 1] : 0ull);
        if (r < j.height) p.row_off[j.row_base + r] = base + incl - v;
        __syncthreads();
        if (tid == 0) s_carry += s_warp[31];
        __syncthreads();
    }
    const unsigned long long end_bit = s_carry;
    const unsigned long long data_bytes = (end_bit + 7 + 7) / 8;  // end-of-block code: 7 zero bits
    const unsigned long long stream_bytes = data_bytes + 4;       // + Adler-32
    const uint32_t chunks = (uint32_t)((stream_bytes + kIdat - 1) / kIdat);
    const uint32_t last_len = (uint32_t)(stream_bytes - (unsigned long long)kIdat * (chunks - 1));
    const unsigned long long file_bytes = kData0 + (unsigned long long)(chunks - 1) * kChunkStride + last_len + 4 + 12;
    const bool error = file_bytes > j.capacity || chunks > j.max_chunks || (stream_bytes + 3) / 4 > j.max_words;
    // Adler-32 of the scanline bytes: a = 1 + sum d, b = N + sum (N - k) d_k over stream
    // byte k; scanline r (bytes k = r*L + i) adds (N - r*L - L) * s0 + s1
    const unsigned long long n_bytes = (unsigned long long)j.height * j.row_bytes;
    unsigned long long a = 0, b = 0;
    for (uint32_t r = tid; r < j.height; r += kLayoutThreads) {
        const unsigned long long s0 = p.s0[j.row_base + r];
        const unsigned long long rest = (n_bytes - (unsigned long long)(r + 1) * j.row_bytes) % kAdlerMod;
        a = (a + s0) % kAdlerMod;
        b = (b + rest * (s0 % kAdlerMod) + p.s1[j.row_base + r] % kAdlerMod) % kAdlerMod;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
        b += __shfl_xor_sync(0xFFFFFFFFu, b, o);
    }
    if (lane == 0) {
        s_a[warp] = a % kAdlerMod;
        s_b[warp] = b % kAdlerMod;
    }
    __syncthreads();
    if (error) {
        if (tid == 0) {
            p.layout[blockIdx.x] = PngLayout{end_bit, stream_bytes, chunks, 0u, 1u, 0u};
            *j.size = 0ull;
        }
        return;
    }
    // IDAT chunk headers (length, type)
    for (uint32_t c = tid; c < chunks; c += kLayoutThreads) {
        uint8_t* h = j.out + kData0 + (size_t)c * kChunkStride - 8;
        put_be32(h, c + 1 < chunks ? kIdat : last_len);
        h[4] = 'I'; h[5] = 'D'; h[6] = 'A'; h[7] = 'T';
    }
    if (tid != 0) return;
    unsigned long long at = 0, bt = 0;
    for (int k = 0; k < kLayoutThreads / 32; ++k) {
        at += s_a[k];
        bt += s_b[k];
    }
    const uint32_t adler_a = (uint32_t)((1 + at) % kAdlerMod);
    const uint32_t adler_b = (uint32_t)((n_bytes % kAdlerMod + bt) % kAdlerMod);
    uint8_t* o = j.out;
    // signature, IHDR, tEXt
    const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    for (int k = 0; k < 8; ++k) o[k] = sig[k];
    uint8_t* ih = o + 8;
    put_be32(ih, 13);
    ih[4] = 'I'; ih[5] = 'H'; ih[6] = 'D'; ih[7] = 'R';
    put_be32(ih + 8, j.width);
    put_be32(ih + 12, j.height);
    ih[16] = 8;                          // bit depth
    ih[17] = j.channels == 4 ? 6 : 2;    // colour type: RGBA / RGB
    ih[18] = 0; ih[19] = 0; ih[20] = 0;  // deflate, adaptive filtering, no interlace
    seal_chunk(s_table, ih, 13);
    uint8_t* tx = o + 33;
    const char text[] = "tEXtSoftware\0AxiomR GB300 frame";  // 27 data bytes after the type
    put_be32(tx, 27);
    for (int k = 0; k < 31; ++k) tx[4 + k] = (uint8_t)text[k];
    seal_chunk(s_table, tx, 27);
    // IEND after the last chunk's CRC
    uint8_t* ie = o + kData0 + (size_t)(chunks - 1) * kChunkStride + last_len + 4;
    put_be32(ie, 0);
    ie[4] = 'I'; ie[5] = 'E'; ie[6] = 'N'; ie[7] = 'D';
    seal_chunk(s_table, ie, 0);
    p.layout[blockIdx.x] = PngLayout{end_bit, stream_bytes, chunks, (adler_b << 16) | adler_a, 0u, 0u};
    *j.size = file_bytes;
}

// bits [b, b + n) (n <= 32) of a staged scanline
__device__ __forceinline__ uint32_t staged_bits(const uint32_t* __restrict__ slot, uint32_t b, uint32_t n) {
    const uint32_t k = b >> 5, sh = b & 31u;
    const unsigned long long two = (unsigned long long)__ldg(slot + k) | ((unsigned long long)__ldg(slot + k + 1) << 32);
    const uint32_t v = (uint32_t)(two >> sh);
    return n >= 32 ? v : (v & ((1u << n) - 1u));
}

// One block per group of 8 scanlines of one image. The block writes the stream words
// that start inside the group's bits (the last group also the tail: end-of-block code,
// padding, Adler-32), each from the zlib and block headers (bits 0-18), the staged bits of
// the scanlines it covers and zeros. The group's scanline offsets sit in shared memory; a
// word that reaches into the next group reads that scanline's offset from global memory.
__global__ void __launch_bounds__(256, 6) png_pack_kernel(const __grid_constant__ PngParams p) {
    __shared__ unsigned long long s_off[kGroupRows + 1];
    __shared__ uint32_t s_bits[kGroupRows];
    const uint2 g = p.groups[blockIdx.x];
    const PngLayout& L = p.layout[g.x];
    if (L.error) return;
    const PngJob& j = p.jobs[g.x];
    const uint32_t r0 = g.y, nr = min(kGroupRows, j.height - r0);
    const unsigned long long* off = p.row_off + j.row_base;
    const uint32_t* bits = p.row_bits + j.row_base;
    const int tid = threadIdx.x;
    if ((uint32_t)tid < nr) {
        s_off[tid] = off[r0 + tid];
        s_bits[tid] = bits[r0 + tid];
    }
    if (tid == 0) s_off[nr] = r0 + nr < j.height ? off[r0 + nr] : L.end_bit;
    __syncthreads();
    const unsigned long long words = (L.stream_bytes + 3) / 4, data_bytes = L.stream_bytes - 4;
    const bool last = r0 + nr >= j.height;
    const unsigned long long w_lo = r0 == 0 ? 0ull : (s_off[0] + 31) / 32;
    const unsigned long long w_hi = last ? words : (s_off[nr] + 31) / 32;
    uint32_t k = 0;  // this thread's scanline (local index), advanced as its words advance
    for (unsigned long long w = w_lo + (unsigned long long)tid; w < w_hi; w += 256) {
        const unsigned long long b0 = w * 32, b1 = b0 + 32;
        uint32_t word = w == 0 ? (0x78u | (0x01u << 8) | (0x3u << 16)) : 0u;
        if (b0 < L.end_bit) {
            while (k + 1 < nr && s_off[k + 1] <= b0) ++k;
            for (uint32_t rr = k;; ++rr) {
                const uint32_t row = r0 + rr;
                if (row >= j.height) break;
                const unsigned long long rs = rr < nr ? s_off[rr] : off[row];
                if (rs >= b1) break;
                const unsigned long long re = rs + (rr < nr ? s_bits[rr] : bits[row]);
                const unsigned long long s = rs > b0 ? rs : b0, e = re < b1 ? re : b1;
                if (e <= s) continue;
                const uint32_t* slot_words = p.stage + j.stage_base + (size_t)row * j.row_words;
                word |= staged_bits(slot_words, (uint32_t)(s - rs), (uint32_t)(e - s)) << (uint32_t)(s - b0);
            }
        }
        if (w * 4 + 4 > data_bytes) {  // Adler-32, most significant byte first, after the data
            for (int q = 0; q < 4; ++q) {
                const unsigned long long byte = w * 4 + q;
                if (byte >= data_bytes && byte < L.stream_bytes) {
                    const uint32_t v = (L.adler >> (24 - 8 * (uint32_t)(byte - data_bytes))) & 255u;
                    word = (word & ~(255u << (8 * q))) | (v << (8 * q));
                }
            }
        }
        *reinterpret_cast<uint32_t*>(j.out + stream_offset(w * 4)) = word;
    }
}

// a * b mod P, bit-reflected (bit 31 holds x^0)
__device__ __forceinline__ uint32_t gf_mul(uint32_t a, uint32_t b) {
    uint32_t prod = 0;
    for (int i = 0; i < 32; ++i) {
        if (a & (0x80000000u >> i)) prod ^= b;
        b = (b >> 1) ^ ((b & 1u) ? kCrcPoly : 0u);  // b * x
    }
    return prod;
}

// x^(8 n) mod P from the table of x^(2^k)
__device__ __forceinline__ uint32_t gf_shift_bytes(const uint32_t* xpow, unsigned long long n) {
    unsigned long long e = n * 8;
    uint32_t r = 0x80000000u;  // x^0
    for (int k = 0; e; ++k, e >>= 1)
        if (e & 1u) r = gf_mul(r, xpow[k]);
    return r;
}

// One block per IDAT chunk; the blocks walk the chunks of all images in order (image by
// image, so no block is launched for a chunk that does not exist). Thread t takes bytes
// [256 t, 256 (t + 1)) of the chunk's type + data as a CRC with zero initial value, four
// bytes per step (slicing by 4: tables T1..T3 derived from T0), then shifts it past the
// bytes after its part (x^(8 a) mod P: a table for full chunks, powers of x^(2^k) for the
// last one); the initial value 0xFFFFFFFF contributes x^(8 total) times itself.
__global__ void __launch_bounds__(256) png_crc_kernel(const __grid_constant__ PngParams p) {
    __shared__ uint32_t s_t[4][256];
    __shared__ uint32_t s_xpow[32];
    __shared__ uint32_t s_part[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    s_t[0][tid] = p.crc_table[tid];
    if (tid < 32) s_xpow[tid] = p.xpow[tid];
    __syncthreads();
    for (int t = 1; t < 4; ++t) {
        const uint32_t c = s_t[t - 1][tid];
        s_t[t][tid] = (c >> 8) ^ s_t[0][c & 255u];
        __syncthreads();
    }
    // chunks before each image (exclusive prefix) for images [tile, tile + kCrcJobs), and
    // the end of the tile; every block walks the same tiles in order
    __shared__ unsigned long long s_before[kCrcJobs + 1];
    __shared__ unsigned long long s_w[8];
    auto load_tile = [&](uint32_t first, unsigned long long before) {
        __syncthreads();  // the previous tile is no longer read
        const uint32_t n = min(kCrcJobs, p.jobs_n - first);
        constexpr int kPer = kCrcJobs / 256;
        uint32_t cnt[kPer];  // this thread's images
        unsigned long long mine = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const uint32_t i = (uint32_t)tid * kPer + q;
            cnt[q] = 0;
            if (i < n) {
                const PngLayout& L = p.layout[first + i];
                cnt[q] = L.error ? 0u : L.chunks;
            }
            mine += cnt[q];
        }
        unsigned long long incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_w[warp] = incl;
        __syncthreads();
        unsigned long long run = before + incl - mine;
        for (int q = 0; q < warp; ++q) run += s_w[q];
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const uint32_t i = (uint32_t)tid * kPer + q;
            if (i < n) s_before[i] = run;
            run += cnt[q];
        }
        if ((uint32_t)tid == (n - 1) / kPer) s_before[n] = run;  // images past n added nothing
        __syncthreads();
    };
    uint32_t tile = 0;
    load_tile(0, 0);
    for (unsigned long long item = blockIdx.x;; item += gridDim.x) {
        uint32_t nt = min(kCrcJobs, p.jobs_n - tile);
        while (item >= s_before[nt] && tile + nt < p.jobs_n) {
            const unsigned long long end = s_before[nt];
            tile += nt;
            load_tile(tile, end);
            nt = min(kCrcJobs, p.jobs_n - tile);
        }
        if (item >= s_before[nt]) break;  // past the last chunk
        // the image of this item: the last one whose first chunk is <= item (images with no
        // chunks share their first-chunk index with the next one)
        uint32_t lo = 0, hi = nt;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_before[mid] <= item) lo = mid; else hi = mid;
        }
        const uint32_t job = tile + lo;
        const unsigned long long first_chunk = s_before[lo];
        const PngLayout& L = p.layout[job];
        const uint32_t c = (uint32_t)(item - first_chunk);
        uint8_t* out = p.jobs[job].out;
        const uint32_t len = c + 1 < L.chunks ? kIdat : (uint32_t)(L.stream_bytes - (unsigned long long)kIdat * c);
        const uint8_t* start = out + kData0 + (size_t)c * kChunkStride - 4;  // type + data, 4-byte aligned
        const uint32_t total = len + 4;
        const uint32_t b0 = min(total, 256u * (uint32_t)tid), b1 = min(total, b0 + 256u);
        uint32_t crc = 0;
        uint32_t k = b0;
        const uint32_t* wp = reinterpret_cast<const uint32_t*>(start);
        for (; k + 16 <= b1; k += 16) {
            const uint32_t w0 = wp[k / 4], w1 = wp[k / 4 + 1], w2 = wp[k / 4 + 2], w3 = wp[k / 4 + 3];
            crc ^= w0;
            crc = s_t[3][crc & 255u] ^ s_t[2][(crc >> 8) & 255u] ^ s_t[1][(crc >> 16) & 255u] ^ s_t[0][crc >> 24];
            crc ^= w1;
            crc = s_t[3][crc & 255u] ^ s_t[2][(crc >> 8) & 255u] ^ s_t[1][(crc >> 16) & 255u] ^ s_t[0][crc >> 24];
            crc ^= w2;
            crc = s_t[3][crc & 255u] ^ s_t[2][(crc >> 8) & 255u] ^ s_t[1][(crc >> 16) & 255u] ^ s_t[0][crc >> 24];
            crc ^= w3;
            crc = s_t[3][crc & 255u] ^ s_t[2][(crc >> 8) & 255u] ^ s_t[1][(crc >> 16) & 255u] ^ s_t[0][crc >> 24];
        }
        for (; k < b1; ++k) crc = s_t[0][(crc ^ start[k]) & 255u] ^ (crc >> 8);
        uint32_t part = 0;
        if (total == kIdat + 4) {  // a full chunk: the shifts are constants
            part = gf_mul(crc, p.full_shift[tid]);
            if (tid == 0) part ^= p.full_init;
        } else {
            if (b1 > b0) part = gf_mul(crc, gf_shift_bytes(s_xpow, total - b1));
            if (tid == 0) part ^= gf_mul(0xFFFFFFFFu, gf_shift_bytes(s_xpow, total));
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) part ^= __shfl_xor_sync(0xFFFFFFFFu, part, o);
        if (lane == 0) s_part[warp] = part;
        __syncthreads();
        if (tid == 0) {
            uint32_t v = 0xFFFFFFFFu;
            for (int q = 0; q < 8; ++q) v ^= s_part[q];
            uint8_t* o = out + kData0 + (size_t)c * kChunkStride + len;
            o[0] = (uint8_t)(v >> 24);
            o[1] = (uint8_t)(v >> 16);
            o[2] = (uint8_t)(v >> 8);
            o[3] = (uint8_t)v;
        }
        __syncthreads();  // s_part is rewritten by the next chunk
    }
}

}  // namespace axr

// ------------------------------------------------------------------ host side

using namespace axr;

namespace {

struct Tables {
    uint32_t crc[256];
    uint32_t xpow[32];
    uint32_t full_shift[256];
    uint32_t full_init;
    Tables() {
        for (uint32_t n = 0; n < 256; ++n) {
            uint32_t c = n;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? (c >> 1) ^ kCrcPoly : c >> 1;
            crc[n] = c;
        }
        auto mul = [](uint32_t a, uint32_t b) {
            uint32_t prod = 0;
            for (int i = 0; i < 32; ++i) {
                if (a & (0x80000000u >> i)) prod ^= b;
                b = (b >> 1) ^ ((b & 1u) ? kCrcPoly : 0u);
            }
            return prod;
        };
        xpow[0] = 0x40000000u;  // x^1
        for (int k = 1; k < 32; ++k) xpow[k] = mul(xpow[k - 1], xpow[k - 1]);
        auto shift = [&](uint64_t bytes) {  // x^(8 bytes)
            uint64_t e = bytes * 8;
            uint32_t r = 0x80000000u;
            for (int k = 0; e; ++k, e >>= 1)
                if (e & 1u) r = mul(r, xpow[k]);
            return r;
        };
        const uint32_t total = kIdat + 4;
        for (uint32_t t = 0; t < 256; ++t) {
            const uint32_t b1 = std::min(total, 256u * (t + 1));
            full_shift[t] = shift(total - b1);
        }
        full_init = mul(0xFFFFFFFFu, shift(total));
    }
};

const Tables& tables() {
    static const Tables t;
    return t;
}

uint64_t row_bytes_of(uint32_t w, uint32_t ch) { return 1ull + (uint64_t)w * ch; }

}  // namespace

namespace {
void release_batch(axr_png_batch* b);
}

namespace axr_internal {

// Scanline scratch, the job table and the pinned staging of axr_framebuffers_encode_png,
// plus the device file buffers and pinned sizes of axr_framebuffers_read_png.
struct PngState {
    uint32_t row_cap = 0, job_cap = 0;
    size_t stage_cap = 0;  // words
    uint32_t* stage = nullptr;
    uint32_t* row_bits = nullptr;
    uint32_t* s0 = nullptr;
    unsigned long long* s1 = nullptr;
    unsigned long long* row_off = nullptr;
    PngJob* jobs = nullptr;
    PngLayout* layout = nullptr;
    uint32_t group_cap = 0;
    uint2* groups = nullptr;
    // pinned host tables, two used in turn so that a call does not wait for the upload of
    // the one before (that upload sits behind the work already on the stream)
    PngJob* jobs_host[2] = {};
    uint2* groups_host[2] = {};
    cudaEvent_t tables_free[2] = {};
    int next = 0;
    axr_png_batch* readback = nullptr;  // axr_framebuffers_read_png
    std::mutex readback_mu;             // held for a whole axr_framebuffers_read_png call
};

void free_png(axr_context* ctx) {
    PngState* s = ctx->png;
    if (!s) return;
    dfree(s->stage);
    dfree(s->row_bits);
    dfree(s->s0);
    dfree(s->s1);
    dfree(s->row_off);
    dfree(s->jobs);
    dfree(s->layout);
    dfree(s->groups);
    for (int t = 0; t < 2; ++t) {
        if (s->groups_host[t]) cudaFreeHost(s->groups_host[t]);
        if (s->jobs_host[t]) cudaFreeHost(s->jobs_host[t]);
        if (s->tables_free[t]) cudaEventDestroy(s->tables_free[t]);
    }
    if (s->readback) release_batch(s->readback);
    delete s;
    ctx->png = nullptr;
}

}  // namespace axr_internal

namespace {

// staging words per scanline: its worst case (filter byte + 9 bits per byte) + one word
// that the pack pass may read past the end
uint32_t row_words_of(uint32_t w, uint32_t ch) {
    return (uint32_t)((8 + 9ull * w * ch + 31) / 32 + 1);
}

axr_status grow_png(axr_context* ctx, uint32_t rows, uint32_t jobs, size_t stage_words, uint32_t groups) {
    if (!ctx->png) ctx->png = new PngState();
    PngState* s = ctx->png;
    for (int t = 0; t < 2; ++t)
        if (!s->tables_free[t]) AXR_CUDA(ctx, cudaEventCreateWithFlags(&s->tables_free[t], cudaEventDisableTiming));
    if (rows > s->row_cap) {
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dfree(s->row_bits); dfree(s->s0); dfree(s->s1); dfree(s->row_off);
        s->row_bits = nullptr; s->s0 = nullptr; s->s1 = nullptr; s->row_off = nullptr;
        s->row_cap = 0;
        const uint32_t cap = std::max(rows, 4096u);
        AXR_CUDA(ctx, dmalloc(&s->row_bits, cap));
        AXR_CUDA(ctx, dmalloc(&s->s0, cap));
        AXR_CUDA(ctx, dmalloc(&s->s1, cap));
        AXR_CUDA(ctx, dmalloc(&s->row_off, cap));
        s->row_cap = cap;
    }
    if (stage_words > s->stage_cap) {
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dfree(s->stage);
        s->stage = nullptr;
        s->stage_cap = 0;
        AXR_CUDA(ctx, dmalloc(&s->stage, stage_words));
        s->stage_cap = stage_words;
    }
    if (groups > s->group_cap) {
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dfree(s->groups);
        s->groups = nullptr;
        for (int t = 0; t < 2; ++t) {
            if (s->groups_host[t]) cudaFreeHost(s->groups_host[t]);
            s->groups_host[t] = nullptr;
        }
        s->group_cap = 0;
        const uint32_t cap = std::max(groups, 1024u);
        AXR_CUDA(ctx, dmalloc(&s->groups, cap));
        for (int t = 0; t < 2; ++t)
            AXR_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&s->groups_host[t]), sizeof(uint2) * cap));
        s->group_cap = cap;
    }
    if (jobs > s->job_cap) {
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dfree(s->jobs); dfree(s->layout);
        s->jobs = nullptr; s->layout = nullptr;
        for (int t = 0; t < 2; ++t) {
            if (s->jobs_host[t]) cudaFreeHost(s->jobs_host[t]);
            s->jobs_host[t] = nullptr;
        }
        s->job_cap = 0;
        const uint32_t cap = std::max(jobs, 64u);
        AXR_CUDA(ctx, dmalloc(&s->jobs, cap));
        AXR_CUDA(ctx, dmalloc(&s->layout, cap));
        for (int t = 0; t < 2; ++t)
            AXR_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&s->jobs_host[t]), sizeof(PngJob) * cap));
        s->job_cap = cap;
    }
    return AXR_OK;
}

// The encode of `count` framebuffers into device buffers; the caller holds ctx->mu.
axr_status encode_locked(axr_context* ctx, int32_t count, const axr_framebuffer* const* fbs, uint32_t channels,
                         void* const* out, const uint64_t* capacity, unsigned long long* sizes) {
    if (channels != 3 && channels != 4) return fail(ctx, AXR_E_INVALID, "channels must be 3 (RGB) or 4 (RGBA)");
    if (count < 0 || (count > 0 && (!fbs || !out || !capacity || !sizes)))
        return fail(ctx, AXR_E_INVALID, "bad framebuffer or buffer list");
    if (count == 0) return AXR_OK;
    uint64_t rows = 0, groups = 0;
    size_t stage_words = 0;
    for (int32_t i = 0; i < count; ++i) {
        const axr_framebuffer* fb = fbs[i];
        if (!fb) return fail(ctx, AXR_E_INVALID, "framebuffer %d is NULL", i);
        if (fb->device != ctx->device) return fail(ctx, AXR_E_INVALID, "framebuffer %d is on another device", i);
        if (!out[i] || (reinterpret_cast<uintptr_t>(out[i]) & 15u))
            return fail(ctx, AXR_E_INVALID, "output buffer %d is NULL or not 16-byte aligned", i);
        const uint64_t bound = axr_png_bound((uint32_t)fb->width, (uint32_t)fb->height, channels);
        if (capacity[i] < bound)
            return fail(ctx, AXR_E_INVALID, "output buffer %d holds %llu bytes, the encode may need %llu", i,
                        (unsigned long long)capacity[i], (unsigned long long)bound);
        rows += (uint64_t)fb->height;
        groups += ((uint64_t)fb->height + kGroupRows - 1) / kGroupRows;
        stage_words += (size_t)fb->height * row_words_of((uint32_t)fb->width, channels);
    }
    if (rows > 0xFFFFFFFFull || count > 65535) return fail(ctx, AXR_E_INVALID, "too many scanlines or images in one call");
    axr_status st = grow_png(ctx, (uint32_t)rows, (uint32_t)count, stage_words + 64, (uint32_t)groups);
    if (st != AXR_OK) return st;
    PngState* s = ctx->png;
    const int tb = s->next;
    s->next ^= 1;
    AXR_CUDA(ctx, cudaEventSynchronize(s->tables_free[tb]));  // the upload two calls ago has been read
    PngJob* jobs_host = s->jobs_host[tb];
    uint2* groups_host = s->groups_host[tb];
    uint32_t row = 0;
    unsigned long long stage = 0;
    for (int32_t i = 0; i < count; ++i) {
        const axr_framebuffer* fb = fbs[i];
        PngJob& j = jobs_host[i];
        const uint64_t bound = axr_png_bound((uint32_t)fb->width, (uint32_t)fb->height, channels);
        j.color = fb->color;
        j.out = static_cast<uint8_t*>(out[i]);
        j.size = sizes + i;
        j.capacity = capacity[i];
        j.width = (uint32_t)fb->width;
        j.height = (uint32_t)fb->height;
        j.channels = channels;
        j.row_bytes = (uint32_t)row_bytes_of(j.width, channels);
        j.row_words = row_words_of(j.width, channels);
        j.stage_base = stage;
        j.row_base = row;
        j.max_chunks = (uint32_t)((bound - kData0 - 16) / kChunkStride);
        j.max_words = ((unsigned long long)j.max_chunks * kIdat + 3) / 4;
        row += j.height;
        stage += (unsigned long long)j.height * j.row_words;
    }
    uint32_t ng = 0;
    for (int32_t i = 0; i < count; ++i)
        for (uint32_t r = 0; r < jobs_host[i].height; r += kGroupRows) groups_host[ng++] = make_uint2((uint32_t)i, r);
    AXR_CUDA(ctx, cudaMemcpyAsync(s->jobs, jobs_host, sizeof(PngJob) * (size_t)count, cudaMemcpyHostToDevice, ctx->stream));
    AXR_CUDA(ctx, cudaMemcpyAsync(s->groups, groups_host, sizeof(uint2) * ng, cudaMemcpyHostToDevice, ctx->stream));
    AXR_CUDA(ctx, cudaEventRecord(s->tables_free[tb], ctx->stream));
    PngParams p{};
    p.jobs = s->jobs;
    p.layout = s->layout;
    p.stage = s->stage;
    p.row_bits = s->row_bits;
    p.s0 = s->s0;
    p.s1 = s->s1;
    p.row_off = s->row_off;
    p.jobs_n = (uint32_t)count;
    p.rows = row;
    std::memcpy(p.crc_table, tables().crc, sizeof(p.crc_table));
    std::memcpy(p.xpow, tables().xpow, sizeof(p.xpow));
    std::memcpy(p.full_shift, tables().full_shift, sizeof(p.full_shift));
    p.full_init = tables().full_init;
    p.groups = s->groups;
    const unsigned row_blocks = (row + kPngWarps - 1) / kPngWarps;
    if (channels == 4) png_rows_kernel<4><<<row_blocks, 32 * kPngWarps, 0, ctx->stream>>>(p);
    else png_rows_kernel<3><<<row_blocks, 32 * kPngWarps, 0, ctx->stream>>>(p);
    AXR_CUDA(ctx, cudaGetLastError());
    png_layout_kernel<<<(unsigned)count, kLayoutThreads, 0, ctx->stream>>>(p);
    AXR_CUDA(ctx, cudaGetLastError());
    png_pack_kernel<<<ng, 256, 0, ctx->stream>>>(p);
    AXR_CUDA(ctx, cudaGetLastError());
    int sms = 0;
    AXR_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    png_crc_kernel<<<(unsigned)sms * 8u, 256, 0, ctx->stream>>>(p);
    AXR_CUDA(ctx, cudaGetLastError());
    ctx->launches += 4;
    return AXR_OK;
}

}  // namespace

extern "C" uint64_t axr_png_bound(uint32_t width, uint32_t height, uint32_t channels) {
    if (width == 0 || height == 0 || (channels != 3 && channels != 4)) return 0;
    // a literal costs at most 9 bits and a match is taken only when it costs fewer bits
    // than the literals it replaces
    const uint64_t bits = kHeaderBits + (uint64_t)height * (8 + 9 * (uint64_t)width * channels);
    const uint64_t stream = (bits + 7 + 7) / 8 + 4;
    const uint64_t chunks = (stream + kIdat - 1) / kIdat;
    return kData0 + chunks * kChunkStride + 16;
}

extern "C" axr_status axr_framebuffers_encode_png(axr_context* ctx, int32_t count, const axr_framebuffer* const* fbs,
                                                  uint32_t channels, void* const* out, const uint64_t* capacity,
                                                  uint64_t* sizes) {
    NvtxRange nvtx_range("axr_framebuffers_encode_png");
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    static_assert(sizeof(uint64_t) == sizeof(unsigned long long), "size array element");
    return encode_locked(ctx, count, fbs, channels, out, capacity, reinterpret_cast<unsigned long long*>(sizes));
}

// A set of PNG files on the device, their sizes copied to pinned memory after the
// encode, and its own copy streams, so that the files of one batch come back to the host
// while the next batch renders and encodes on the context stream.
struct axr_png_batch {
    int device = 0;
    uint8_t* files = nullptr;
    size_t files_cap = 0;
    unsigned long long* sizes_dev = nullptr;
    unsigned long long* sizes_host = nullptr;  // pinned
    uint32_t sizes_cap = 0;
    std::vector<size_t> at;  // file i at files + at[i]
    int32_t count = 0;
    bool encoded = false;
    cudaEvent_t done = nullptr;  // the sizes are on the host (context stream)
    static constexpr int kStreams = 4;
    cudaStream_t copy[kStreams] = {};
    cudaEvent_t copied[kStreams] = {};
};

namespace {

void release_batch(axr_png_batch* b) {
    for (int k = 0; k < axr_png_batch::kStreams; ++k) {
        if (b->copy[k]) {
            cudaStreamSynchronize(b->copy[k]);
            cudaStreamDestroy(b->copy[k]);
        }
        if (b->copied[k]) cudaEventDestroy(b->copied[k]);
    }
    if (b->done) {
        cudaEventSynchronize(b->done);
        cudaEventDestroy(b->done);
    }
    dfree(b->files);
    dfree(b->sizes_dev);
    if (b->sizes_host) cudaFreeHost(b->sizes_host);
    delete b;
}

axr_status create_batch(axr_context* ctx, axr_png_batch** out) {
    axr_png_batch* b = new axr_png_batch();
    b->device = ctx->device;
    cudaError_t e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    for (int k = 0; e == cudaSuccess && k < axr_png_batch::kStreams; ++k) {
        e = cudaStreamCreateWithFlags(&b->copy[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->copied[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        release_batch(b);
        return cuda_fail(ctx, e, "PNG batch streams");
    }
    *out = b;
    return AXR_OK;
}

// Enqueue the encode of `count` framebuffers into b on the context stream, then the copy
// of the sizes; the caller holds ctx->mu.
axr_status batch_encode_locked(axr_context* ctx, axr_png_batch* b, int32_t count, const axr_framebuffer* const* fbs,
                               uint32_t channels) {
    if (channels != 3 && channels != 4) return fail(ctx, AXR_E_INVALID, "channels must be 3 (RGB) or 4 (RGBA)");
    if (count < 0 || (count > 0 && !fbs)) return fail(ctx, AXR_E_INVALID, "bad framebuffer list");
    std::vector<uint64_t> cap((size_t)count);
    b->at.assign((size_t)count + 1, 0);
    for (int32_t i = 0; i < count; ++i) {
        if (!fbs[i]) return fail(ctx, AXR_E_INVALID, "framebuffer %d is NULL", i);
        cap[i] = axr_png_bound((uint32_t)fbs[i]->width, (uint32_t)fbs[i]->height, channels);
        b->at[i + 1] = b->at[i] + ((cap[i] + 255) & ~uint64_t(255));
    }
    // the batch's earlier files must have been copied out before they are overwritten
    for (int k = 0; k < axr_png_batch::kStreams; ++k) AXR_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, b->copied[k], 0));
    if (b->at[count] > b->files_cap) {
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dfree(b->files);
        b->files = nullptr;
        b->files_cap = 0;
        AXR_CUDA(ctx, dmalloc(&b->files, b->at[count]));
        b->files_cap = b->at[count];
    }
    if ((uint32_t)count > b->sizes_cap) {
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dfree(b->sizes_dev);
        b->sizes_dev = nullptr;
        if (b->sizes_host) cudaFreeHost(b->sizes_host);
        b->sizes_host = nullptr;
        b->sizes_cap = 0;
        AXR_CUDA(ctx, dmalloc(&b->sizes_dev, (size_t)count));
        AXR_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&b->sizes_host), sizeof(unsigned long long) * count));
        b->sizes_cap = (uint32_t)count;
    }
    b->count = count;
    b->encoded = false;
    if (count == 0) return AXR_OK;
    std::vector<void*> out((size_t)count);
    for (int32_t i = 0; i < count; ++i) out[i] = b->files + b->at[i];
    axr_status st = encode_locked(ctx, count, fbs, channels, out.data(), cap.data(), b->sizes_dev);
    if (st != AXR_OK) return st;
    AXR_CUDA(ctx, cudaMemcpyAsync(b->sizes_host, b->sizes_dev, sizeof(unsigned long long) * count,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    AXR_CUDA(ctx, cudaEventRecord(b->done, ctx->stream));
    b->encoded = true;
    return AXR_OK;
}

axr_status batch_sizes(axr_context* ctx, axr_png_batch* b, uint64_t* sizes) {
    if (!b->encoded) return b->count == 0 ? AXR_OK : fail(ctx, AXR_E_INVALID, "the PNG batch holds no encode");
    DeviceGuard g(b->device);
    AXR_CUDA(ctx, cudaEventSynchronize(b->done));
    for (int32_t i = 0; i < b->count; ++i) {
        if (b->sizes_host[i] == 0) return fail(ctx, AXR_E_CUDA, "framebuffer %d: encode overflow", i);
        if (sizes) sizes[i] = b->sizes_host[i];
    }
    return AXR_OK;
}

axr_status batch_read(axr_context* ctx, axr_png_batch* b, void* const* files, const uint64_t* capacity) {
    axr_status st = batch_sizes(ctx, b, nullptr);
    if (st != AXR_OK || b->count == 0) return st;
    if (!files) return fail(ctx, AXR_E_INVALID, "no host buffers");
    for (int32_t i = 0; i < b->count; ++i)
        if (files[i] && capacity && capacity[i] < b->sizes_host[i])
            return fail(ctx, AXR_E_INVALID, "host buffer %d holds %llu bytes, the file has %llu", i,
                        (unsigned long long)capacity[i], b->sizes_host[i]);
    DeviceGuard g(b->device);
    for (int k = 0; k < axr_png_batch::kStreams; ++k) AXR_CUDA(ctx, cudaStreamWaitEvent(b->copy[k], b->done, 0));
    for (int32_t i = 0; i < b->count; ++i) {
        if (!files[i]) continue;
        AXR_CUDA(ctx, cudaMemcpyAsync(files[i], b->files + b->at[i], b->sizes_host[i], cudaMemcpyDeviceToHost,
                                      b->copy[i % axr_png_batch::kStreams]));
    }
    for (int k = 0; k < axr_png_batch::kStreams; ++k) AXR_CUDA(ctx, cudaEventRecord(b->copied[k], b->copy[k]));
    for (int k = 0; k < axr_png_batch::kStreams; ++k) AXR_CUDA(ctx, cudaEventSynchronize(b->copied[k]));
    return AXR_OK;
}

}  // namespace

namespace axr_internal {

axr_status png_batch_create(axr_context* ctx, axr_png_batch** out) { return create_batch(ctx, out); }

void png_batch_release(axr_png_batch* b) {
    if (b) release_batch(b);
}

axr_status png_batch_encode_locked(axr_context* ctx, axr_png_batch* b, int32_t count,
                                   const axr_framebuffer* const* fbs, uint32_t channels) {
    return batch_encode_locked(ctx, b, count, fbs, channels);
}

cudaError_t png_batch_query(const axr_png_batch* b) {
    return b->encoded ? cudaEventQuery(b->done) : cudaSuccess;
}

void png_batch_file(const axr_png_batch* b, int32_t i, const void** dev, uint64_t* size) {
    *dev = b->files + b->at[(size_t)i];
    *size = b->sizes_host[i];
}

}  // namespace axr_internal

extern "C" axr_status axr_png_batch_create(axr_context* ctx, axr_png_batch** out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    return create_batch(ctx, out);
}

extern "C" void axr_png_batch_destroy(axr_context* ctx, axr_png_batch* b) {
    if (!b) return;
    DeviceGuard g(b->device);
    release_batch(b);
}

extern "C" axr_status axr_png_batch_encode(axr_context* ctx, axr_png_batch* b, int32_t count,
                                           const axr_framebuffer* const* fbs, uint32_t channels) {
    NvtxRange nvtx_range("axr_png_batch_encode");
    if (!ctx || !b) return fail(ctx, AXR_E_INVALID, "NULL argument");
    if (b->device != ctx->device) return fail(ctx, AXR_E_INVALID, "the PNG batch belongs to another device");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    return batch_encode_locked(ctx, b, count, fbs, channels);
}

extern "C" axr_status axr_png_batch_sizes(axr_context* ctx, axr_png_batch* b, uint64_t* sizes) {
    if (!ctx || !b || !sizes) return fail(ctx, AXR_E_INVALID, "NULL argument");
    return batch_sizes(ctx, b, sizes);
}

extern "C" axr_status axr_png_batch_read(axr_context* ctx, axr_png_batch* b, void* const* files,
                                         const uint64_t* capacity) {
    if (!ctx || !b) return fail(ctx, AXR_E_INVALID, "NULL argument");
    return batch_read(ctx, b, files, capacity);
}

extern "C" axr_status axr_framebuffers_read_png(axr_context* ctx, int32_t count, const axr_framebuffer* const* fbs,
                                                uint32_t channels, void* const* files, const uint64_t* capacity,
                                                uint64_t* sizes) {
    NvtxRange nvtx_range("axr_framebuffers_read_png");
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    if (count < 0 || (count > 0 && (!fbs || !sizes))) return fail(ctx, AXR_E_INVALID, "bad framebuffer list");
    if (channels != 3 && channels != 4) return fail(ctx, AXR_E_INVALID, "channels must be 3 (RGB) or 4 (RGBA)");
    if (count == 0) return AXR_OK;
    axr_png_batch* b;
    PngState* ps;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (!ctx->png) ctx->png = new PngState();
        ps = ctx->png;
    }
    // the internal batch serves one call at a time (lock order: readback_mu, then ctx->mu)
    std::lock_guard<std::mutex> whole(ps->readback_mu);
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        DeviceGuard g(ctx->device);
        if (!ctx->png->readback) {
            axr_status st = create_batch(ctx, &ctx->png->readback);
            if (st != AXR_OK) return st;
        }
        b = ctx->png->readback;
        axr_status st = batch_encode_locked(ctx, b, count, fbs, channels);
        if (st != AXR_OK) return st;
    }
    axr_status st = batch_sizes(ctx, b, sizes);
    if (st != AXR_OK || !files) return st;
    for (int32_t i = 0; i < count; ++i)
        if (files[i] && capacity && capacity[i] < sizes[i])
            return fail(ctx, AXR_E_INVALID, "a host buffer is smaller than its file (sizes returned)");
    return batch_read(ctx, b, files, capacity);
}
