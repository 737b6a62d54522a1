// spx_hash.cuh -- register-resident hash cores and SPHINCS+ tweakable hashes
// for sm_103a.
//
// Values (n-byte hash outputs) live in registers as W = n/4 32-bit words in
// the hash family's native order: big-endian words for SHA-256, the
// little-endian memory order for SHAKE-256 (so Keccak lanes are plain 64-bit
// loads).  Addresses (ADRS) are six big-endian words covering bytes 0..23 of
// the reference's 32-byte address; bytes 24..31 are always zero.
//
// Field offsets follow the reference's SHA-256 offset table, which its
// params.h includes for every hash (sha256_offsets.h:9-17): layer @0,
// tree @1..8, type @9, key pair @12..13, chain/height @17, tree index
// @18..21, hash address @21.
#pragma once
#include <stdint.h>

namespace cuspx {

#define SPX_DEV __device__ __forceinline__

enum : uint32_t { ADDR_WOTS = 0, ADDR_WOTSPK = 1, ADDR_HASHTREE = 2, ADDR_FORSTREE = 3, ADDR_FORSPK = 4 };

// ---------------------------------------------------------------------------
// ADRS in six big-endian words (address.cu:10-180)
// ---------------------------------------------------------------------------
struct Adrs {
    uint32_t w[6];
};

SPX_DEV void adrs_zero(Adrs &a) {
#pragma unroll
    for (int i = 0; i < 6; i++) a.w[i] = 0;
}
SPX_DEV void adrs_layer(Adrs &a, uint32_t l) { a.w[0] = (a.w[0] & 0x00ffffffu) | (l << 24); }
SPX_DEV void adrs_tree(Adrs &a, uint64_t t) {
    a.w[0] = (a.w[0] & 0xff000000u) | (uint32_t)(t >> 40);
    a.w[1] = (uint32_t)(t >> 8);
    a.w[2] = (a.w[2] & 0x00ffffffu) | ((uint32_t)t << 24);
}
SPX_DEV void adrs_type(Adrs &a, uint32_t t) { a.w[2] = (a.w[2] & 0xff00ffffu) | (t << 16); }
// The reference writes the key-pair high byte only for subtrees taller than
// 8; a key-pair index below 256 has a zero high byte, so writing both bytes
// always is byte-identical.
SPX_DEV void adrs_keypair(Adrs &a, uint32_t kp) { a.w[3] = (a.w[3] & 0x0000ffffu) | (kp << 16); }
SPX_DEV void adrs_chain(Adrs &a, uint32_t c) { a.w[4] = (a.w[4] & 0xff00ffffu) | (c << 16); }
SPX_DEV void adrs_height(Adrs &a, uint32_t h) { a.w[4] = (a.w[4] & 0xff00ffffu) | (h << 16); }
SPX_DEV void adrs_hash(Adrs &a, uint32_t h) { a.w[5] = (a.w[5] & 0xff00ffffu) | (h << 16); }
SPX_DEV void adrs_index(Adrs &a, uint32_t i) {
    a.w[4] = (a.w[4] & 0xffff0000u) | (i >> 16);
    a.w[5] = (a.w[5] & 0x0000ffffu) | (i << 16);
}
// copy_subtree_addr: bytes 0..8 (layer + tree)
SPX_DEV void adrs_copy_subtree(Adrs &o, const Adrs &i) {
    o.w[0] = i.w[0];
    o.w[1] = i.w[1];
    o.w[2] = (o.w[2] & 0x00ffffffu) | (i.w[2] & 0xff000000u);
}
// copy_keypair_addr: layer + tree + key pair
SPX_DEV void adrs_copy_keypair(Adrs &o, const Adrs &i) {
    adrs_copy_subtree(o, i);
    o.w[3] = (o.w[3] & 0x0000ffffu) | (i.w[3] & 0xffff0000u);
}

SPX_DEV uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// ---------------------------------------------------------------------------
// SHA-256 compression (FIPS 180-4), fully unrolled over 64 rounds with the
// schedule in a rolling 16-word window.  Rotates are single funnel shifts,
// Ch/Maj/three-way xors compile to LOP3.
// ---------------------------------------------------------------------------
// FIPS 180-4 round constants and initial value, returned by constexpr
// functions so that every use in the unrolled rounds folds to an immediate.
__host__ __device__ constexpr uint32_t sha256_k(int i) {
    constexpr uint32_t k[64] = {
        0x428a2f98u, 0x71374491u, 0xb5c0fbcfu, 0xe9b5dba5u, 0x3956c25bu, 0x59f111f1u, 0x923f82a4u, 0xab1c5ed5u,
        0xd807aa98u, 0x12835b01u, 0x243185beu, 0x550c7dc3u, 0x72be5d74u, 0x80deb1feu, 0x9bdc06a7u, 0xc19bf174u,
        0xe49b69c1u, 0xefbe4786u, 0x0fc19dc6u, 0x240ca1ccu, 0x2de92c6fu, 0x4a7484aau, 0x5cb0a9dcu, 0x76f988dau,
        0x983e5152u, 0xa831c66du, 0xb00327c8u, 0xbf597fc7u, 0xc6e00bf3u, 0xd5a79147u, 0x06ca6351u, 0x14292967u,
        0x27b70a85u, 0x2e1b2138u, 0x4d2c6dfcu, 0x53380d13u, 0x650a7354u, 0x766a0abbu, 0x81c2c92eu, 0x92722c85u,
        0xa2bfe8a1u, 0xa81a664bu, 0xc24b8b70u, 0xc76c51a3u, 0xd192e819u, 0xd6990624u, 0xf40e3585u, 0x106aa070u,
        0x19a4c116u, 0x1e376c08u, 0x2748774cu, 0x34b0bcb5u, 0x391c0cb3u, 0x4ed8aa4au, 0x5b9cca4fu, 0x682e6ff3u,
        0x748f82eeu, 0x78a5636fu, 0x84c87814u, 0x8cc70208u, 0x90befffau, 0xa4506cebu, 0xbef9a3f7u, 0xc67178f2u};
    return k[i];
}
__host__ __device__ constexpr uint32_t sha256_iv_word(int i) {
    constexpr uint32_t iv[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                                0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
    return iv[i];
}

SPX_DEV uint32_t rotr(uint32_t x, int c) { return __funnelshift_r(x, x, c); }

// Pipe balancing.  The compression is bound by the ALU pipe (funnel
// shifts, LOP3 and IADD3 all issue there) while the FMA pipe idles.  An add
// written as a * c_one + b with c_one an opaque constant-bank 1 must issue as
// IMAD on the FMA pipe, so the 2-input adds (e = d + t1 each round, the last
// add of each schedule word, the schedule word into t1) move there.
// Shifts and rotates stay on the ALU: as multiplies by 2^(32-k) from the
// constant bank (x >> k = umulhi, rotr = x * m + umulhi) they measured
// slower at every depth tried (k_leaves +0.2% for the sigma shifts alone,
// +28% with five rotates per round moved), as IMAD.HI does not issue at
// IMAD's rate.  CUSPX_FMA_ADDS=0 restores plain adds.
#ifndef CUSPX_FMA_ADDS
#define CUSPX_FMA_ADDS 1
#endif
static __constant__ uint32_t c_one = 1u;
SPX_DEV uint32_t add_fma(uint32_t a, uint32_t b) {
#if CUSPX_FMA_ADDS
    return a * c_one + b;
#else
    return a + b;
#endif
}

// the four SHA-256 sigma functions (FIPS 180-4 4.4-4.7)
SPX_DEV uint32_t sha_Sigma0(uint32_t a) {
    return rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
}
SPX_DEV uint32_t sha_Sigma1(uint32_t e) {
    return rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
}
SPX_DEV uint32_t sha_sigma0(uint32_t x) {
    return rotr(x, 7) ^ rotr(x, 18) ^ (x >> 3);
}
SPX_DEV uint32_t sha_sigma1(uint32_t y) {
    return rotr(y, 17) ^ rotr(y, 19) ^ (y >> 10);
}

SPX_DEV void sha256_iv(uint32_t s[8]) {
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = sha256_iv_word(i);
}

// Rounds [R0, R1) of the compression on the working variables st = a..h;
// w is the rolling 16-word schedule window (overwritten as it expands).
// (Folding d into h + K + W a round early, e' = (d + h + K + W) + Sigma1 + Ch,
// shortens the e chain by one step at one more ALU add a round; it measured
// slower even for a warp alone on its SM: a lone verify 1.14 -> 1.20 ms.)
template <int R0, int R1>
SPX_DEV void sha256_rounds(uint32_t st[8], uint32_t w[16]) {
    uint32_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], h = st[7];
#pragma unroll
    for (int i = R0; i < R1; i++) {
        uint32_t wi;
        if (i < 16) {
            wi = w[i];
        } else {
            wi = w[i & 15] = add_fma(w[i & 15], sha_sigma0(w[(i - 15) & 15]) + w[(i - 7) & 15] +
                                                    sha_sigma1(w[(i - 2) & 15]));
        }
        // h + K is ready a round early, so the schedule word joins it on the FMA pipe
        uint32_t t1 = add_fma(h + sha256_k(i), wi) + sha_Sigma1(e) + ((e & f) ^ (~e & g));
        uint32_t t2 = sha_Sigma0(a) + ((a & b) | (c & (a | b)));
        h = g;
        g = f;
        f = e;
        e = add_fma(d, t1);
        d = c;
        c = b;
        b = a;
        a = t1 + t2;
    }
    st[0] = a; st[1] = b; st[2] = c; st[3] = d; st[4] = e; st[5] = f; st[6] = g; st[7] = h;
}

// Message schedule with the round constants added: kw[t * S] = W_t + K_t
// for t = 0..63 from the 16 block words w (consumed); S interleaves the
// buffers of several threads in shared memory.
template <int S>
SPX_DEV void sha256_schedule_kw(uint32_t *kw, uint32_t w[16]) {
#pragma unroll
    for (int i = 0; i < 64; i++) {
        if (i >= 16) {
            w[i & 15] = w[i & 15] + sha_sigma0(w[(i - 15) & 15]) + w[(i - 7) & 15] + sha_sigma1(w[(i - 2) & 15]);
        }
        kw[i * S] = add_fma(w[i & 15], sha256_k(i));
    }
}

// s <- compress(s) with the schedule given as kw[t * S] = W_t + K_t (the
// rounds alone: the schedule was computed elsewhere)
template <int S>
SPX_DEV void sha256_compress_kw(uint32_t s[8], const uint32_t *kw) {
    uint32_t a = s[0], b = s[1], c = s[2], d = s[3], e = s[4], f = s[5], g = s[6], h = s[7];
#pragma unroll
    for (int i = 0; i < 64; i++) {
        const uint32_t t1 = add_fma(h, kw[i * S]) + sha_Sigma1(e) + ((e & f) ^ (~e & g));
        const uint32_t t2 = sha_Sigma0(a) + ((a & b) | (c & (a | b)));
        h = g;
        g = f;
        f = e;
        e = add_fma(d, t1);
        d = c;
        c = b;
        b = a;
        a = t1 + t2;
    }
    s[0] += a; s[1] += b; s[2] += c; s[3] += d; s[4] += e; s[5] += f; s[6] += g; s[7] += h;
}

// s <- compress(s, w); w is consumed (overwritten by the schedule).
SPX_DEV void sha256_compress(uint32_t s[8], uint32_t w[16]) {
    uint32_t t[8];
#pragma unroll
    for (int i = 0; i < 8; i++) t[i] = s[i];
    sha256_rounds<0, 64>(t, w);
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] += t[i];
}

// ---------------------------------------------------------------------------
// Keccak-f[1600] (FIPS 202) on 25 64-bit lanes held in registers.
// ---------------------------------------------------------------------------
__constant__ static const uint64_t KECCAK_RC[24] = {
    0x0000000000000001ull, 0x0000000000008082ull, 0x800000000000808aull, 0x8000000080008000ull,
    0x000000000000808bull, 0x0000000080000001ull, 0x8000000080008081ull, 0x8000000000008009ull,
    0x000000000000008aull, 0x0000000000000088ull, 0x0000000080008009ull, 0x000000008000000aull,
    0x000000008000808bull, 0x800000000000008bull, 0x8000000000008089ull, 0x8000000000008003ull,
    0x8000000000008002ull, 0x8000000000000080ull, 0x000000000000800aull, 0x800000008000000aull,
    0x8000000080008081ull, 0x8000000000008080ull, 0x0000000080000001ull, 0x8000000080008008ull};

SPX_DEV uint64_t rotl64(uint64_t x, int c) { return (x << c) | (x >> (64 - c)); }
SPX_DEV uint64_t xor5(uint64_t a, uint64_t b, uint64_t c, uint64_t d, uint64_t e) { return a ^ b ^ c ^ d ^ e; }

SPX_DEV void keccak_f1600(uint64_t A[25]) {
#pragma unroll 2
    for (int r = 0; r < 24; r++) {
        // theta
        uint64_t C0 = xor5(A[0], A[5], A[10], A[15], A[20]);
        uint64_t C1 = xor5(A[1], A[6], A[11], A[16], A[21]);
        uint64_t C2 = xor5(A[2], A[7], A[12], A[17], A[22]);
        uint64_t C3 = xor5(A[3], A[8], A[13], A[18], A[23]);
        uint64_t C4 = xor5(A[4], A[9], A[14], A[19], A[24]);
        uint64_t D0 = C4 ^ rotl64(C1, 1), D1 = C0 ^ rotl64(C2, 1), D2 = C1 ^ rotl64(C3, 1);
        uint64_t D3 = C2 ^ rotl64(C4, 1), D4 = C3 ^ rotl64(C0, 1);
        // theta + rho + pi: B[y][2x+3y] = rot(A[x][y] ^ D[x], r[x][y])
        uint64_t B00 = A[0] ^ D0;
        uint64_t B10 = rotl64(A[6] ^ D1, 44);
        uint64_t B20 = rotl64(A[12] ^ D2, 43);
        uint64_t B30 = rotl64(A[18] ^ D3, 21);
        uint64_t B40 = rotl64(A[24] ^ D4, 14);
        uint64_t B01 = rotl64(A[3] ^ D3, 28);
        uint64_t B11 = rotl64(A[9] ^ D4, 20);
        uint64_t B21 = rotl64(A[10] ^ D0, 3);
        uint64_t B31 = rotl64(A[16] ^ D1, 45);
        uint64_t B41 = rotl64(A[22] ^ D2, 61);
        uint64_t B02 = rotl64(A[1] ^ D1, 1);
        uint64_t B12 = rotl64(A[7] ^ D2, 6);
        uint64_t B22 = rotl64(A[13] ^ D3, 25);
        uint64_t B32 = rotl64(A[19] ^ D4, 8);
        uint64_t B42 = rotl64(A[20] ^ D0, 18);
        uint64_t B03 = rotl64(A[4] ^ D4, 27);
        uint64_t B13 = rotl64(A[5] ^ D0, 36);
        uint64_t B23 = rotl64(A[11] ^ D1, 10);
        uint64_t B33 = rotl64(A[17] ^ D2, 15);
        uint64_t B43 = rotl64(A[23] ^ D3, 56);
        uint64_t B04 = rotl64(A[2] ^ D2, 62);
        uint64_t B14 = rotl64(A[8] ^ D3, 55);
        uint64_t B24 = rotl64(A[14] ^ D4, 39);
        uint64_t B34 = rotl64(A[15] ^ D0, 41);
        uint64_t B44 = rotl64(A[21] ^ D1, 2);
        // chi + iota (row y holds lanes A[5y..5y+4])
        A[0] = B00 ^ (~B10 & B20) ^ KECCAK_RC[r];
        A[1] = B10 ^ (~B20 & B30);
        A[2] = B20 ^ (~B30 & B40);
        A[3] = B30 ^ (~B40 & B00);
        A[4] = B40 ^ (~B00 & B10);
        A[5] = B01 ^ (~B11 & B21);
        A[6] = B11 ^ (~B21 & B31);
        A[7] = B21 ^ (~B31 & B41);
        A[8] = B31 ^ (~B41 & B01);
        A[9] = B41 ^ (~B01 & B11);
        A[10] = B02 ^ (~B12 & B22);
        A[11] = B12 ^ (~B22 & B32);
        A[12] = B22 ^ (~B32 & B42);
        A[13] = B32 ^ (~B42 & B02);
        A[14] = B42 ^ (~B02 & B12);
        A[15] = B03 ^ (~B13 & B23);
        A[16] = B13 ^ (~B23 & B33);
        A[17] = B23 ^ (~B33 & B43);
        A[18] = B33 ^ (~B43 & B03);
        A[19] = B43 ^ (~B03 & B13);
        A[20] = B04 ^ (~B14 & B24);
        A[21] = B14 ^ (~B24 & B34);
        A[22] = B24 ^ (~B34 & B44);
        A[23] = B34 ^ (~B44 & B04);
        A[24] = B44 ^ (~B04 & B14);
    }
}

// ---------------------------------------------------------------------------
// Keccak-f[1600] spread over one warp, for the serial sponge of a long
// message: lane i < 25 holds state lane i (x = i % 5, y = i / 5); lanes
// 25..31 compute values nobody reads and only take part in the shuffles.
// A round is 20 32-bit shuffles and ~20 ALU operations on each lane instead
// of ~190 instructions of one thread, so a permutation's latency drops
// while a lone message is hashed.  Same function as keccak_f1600 (FIPS 202).
// ---------------------------------------------------------------------------
// rotation of lane i (rho, by the FIPS 202 recurrence) and the lane whose
// rotated value lands in lane i (pi: A[x + 5y] goes to y + 5((2x + 3y) mod 5))
__constant__ static const uint8_t KECCAK_RHO[32] = {0,  1,  62, 28, 27, 36, 44, 6,  55, 20, 3,
                                                     10, 43, 25, 39, 41, 45, 15, 21, 8,  18, 2,
                                                     61, 56, 14, 0,  0,  0,  0,  0,  0,  0};
__constant__ static const uint8_t KECCAK_PI_SRC[32] = {0,  6,  12, 18, 24, 3,  9,  10, 16, 22, 1,
                                                        7,  13, 19, 20, 4,  5,  11, 17, 23, 2,  8,
                                                        14, 15, 21, 25, 26, 27, 28, 29, 30, 31};

// per-lane constants of warp_keccak_f1600
struct KeccakLane {
    uint32_t col[5];      // lanes of this lane's column (C[x])
    uint32_t xm1, xp1;    // row-0 lanes holding C[x - 1], C[x + 1]
    uint32_t rp1, rp2;    // lanes (x + 1, y), (x + 2, y) of this row (chi)
    uint32_t src;         // pi source lane
    uint32_t swap, s;     // rho: halves swapped when the rotation is >= 32, then s = rotation mod 32
};
SPX_DEV void keccak_lane_init(KeccakLane &k, uint32_t lane) {
    const uint32_t x = lane % 5, y = lane < 25 ? lane / 5 : 0;
#pragma unroll
    for (int yy = 0; yy < 5; yy++) k.col[yy] = x + 5 * yy;
    k.xm1 = (x + 4) % 5;
    k.xp1 = (x + 1) % 5;
    k.rp1 = (x + 1) % 5 + 5 * y;
    k.rp2 = (x + 2) % 5 + 5 * y;
    k.src = KECCAK_PI_SRC[lane];
    const uint32_t r = KECCAK_RHO[lane];
    k.swap = r >= 32;
    k.s = r & 31;
}
SPX_DEV uint64_t shfl64(uint64_t v, uint32_t src) {
    const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
    const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
    return ((uint64_t)hi << 32) | lo;
}
// every lane of the warp calls this (a: this lane's state lane)
SPX_DEV void warp_keccak_f1600(uint64_t &a, const KeccakLane &k, uint32_t lane) {
#pragma unroll 1
    for (int r = 0; r < 24; r++) {
        // theta
        const uint64_t C = shfl64(a, k.col[0]) ^ shfl64(a, k.col[1]) ^ shfl64(a, k.col[2]) ^
                           shfl64(a, k.col[3]) ^ shfl64(a, k.col[4]);
        const uint64_t cp = shfl64(C, k.xp1);
        a ^= shfl64(C, k.xm1) ^ ((cp << 1) | (cp >> 63));
        // rho: rotate left by 32 * swap + s
        uint32_t lo = (uint32_t)a, hi = (uint32_t)(a >> 32);
        const uint32_t l2 = k.swap ? hi : lo, h2 = k.swap ? lo : hi;
        lo = __funnelshift_l(h2, l2, k.s);
        hi = __funnelshift_l(l2, h2, k.s);
        // pi
        const uint64_t b = shfl64(((uint64_t)hi << 32) | lo, k.src);
        // chi + iota
        a = b ^ (~shfl64(b, k.rp1) & shfl64(b, k.rp2));
        if (lane == 0) a ^= KECCAK_RC[r];
    }
}

SPX_DEV uint64_t lane_of(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }

// ADRS as the four little-endian Keccak lanes of its 32 bytes
SPX_DEV void adrs_lanes(const Adrs &a, uint64_t l[4]) {
    l[0] = lane_of(bswap32(a.w[0]), bswap32(a.w[1]));
    l[1] = lane_of(bswap32(a.w[2]), bswap32(a.w[3]));
    l[2] = lane_of(bswap32(a.w[4]), bswap32(a.w[5]));
    l[3] = 0;
}

}  // namespace cuspx
