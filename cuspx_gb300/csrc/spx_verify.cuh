// spx_verify.cuh -- persistent hypertree verify (every parameter set).
//
// crypto_sign_verify (sign.cu:3048-3121) is serial over the d layers of an
// item: layer L's WOTS+ chains (wots_pk_from_sig, wots.cu:777-804) need the
// root of layer L-1, T_len (sign.cu:3103) needs every chain end of layer L,
// and compute_root (utils.cu:94-135) needs T_len.  Per item that is ~10-way
// parallel work on average (len chains, then one serial T_len + auth path),
// so flat per-layer kernels leave the GPU idle during every T phase.
//
// Here one launch runs the whole hypertree for the batch.  Each warp owns G
// item slots in shared memory and keeps every lane busy with whichever task
// any of its items offers:
//
//   chain   one F per iteration, from the signature value to step 15
//   T       one block of T_k (FORS key) or T_len per iteration
//   root    one H of compute_root per iteration (SHA-256 n >= 24: two blocks)
//
// Every task is "one unit of the hash per iteration": a SHA-256 compression
// from a state over a 16-word block, or a Keccak-f[1600] permutation of a
// state with a 17-lane block absorbed.  Lanes differ only in how they build
// the unit's input and use its output, so the hash itself -- the expensive
// part -- runs converged across the warp whatever mix of tasks the lanes
// hold.  Items are taken from a global counter as slots free up, so a batch
// of any size keeps all warps busy.
//
// T streams behind the chains: block j of the T input only needs the chains
// whose end values it covers, so the T lane starts as soon as the first
// block's chains are done and takes each later block once its chains are; on
// an iteration where its next block is not ready it idles.  This shortens an
// item's per-layer critical path from ~15 + |T| + h' to ~15 + 2 + h' units.
//
// Slot data lives in shared memory: the T input stream (prefix || values ||
// padding, memory byte order) into which the layer's WOTS signature is
// copied and where each chain's end value overwrites its start value in
// place, a bit per finished chain, the layer's auth path, the chain lengths,
// the key material and the item's position (SHAKE also keeps the T sponge
// state there).  Slots are private to their warp, so nothing waits on
// another warp; the loop ends when the counter is exhausted and every slot
// is empty.
//
// Items per warp: a small batch is bound by one item's serial path, so the
// host launches one item per warp until there are about 4 warps per SM and
// only then packs up to verify_slots items into a warp.
#pragma once
#include <type_traits>

#include "spx_kernels.cuh"

namespace cuspx {

// Slot layout and bookkeeping shared by both hash families.  PRE is the
// T stream's prefix in bytes (what is hashed before the first value) and
// BLK its block size in bytes.
template <int N_, int PRE, int BLK>
struct VerifySlot {
    static constexpr int N = N_, W = N / 4, LEN = 2 * N + 3;
    // slot header word indices
    enum : int {
        S_ITEM = 0,      // batch index of the item
        S_LAYER,         // -1: T_k over the FORS roots; 0..d-1: WOTS layer
        S_NEXT,          // next chain to hand out
        S_TCLAIM,        // the T stream has a lane
        S_STATE,         // EMPTY / ACTIVE / ADVANCE / DEAD
        S_TREE_LO, S_TREE_HI, S_IDX_LEAF,   // hypertree position from H_msg
        S_IDXL,          // leaf index within the current layer's tree
        S_AW0, S_AW1, S_AW2,                // ADRS words 0..2 of the current layer (type WOTS)
        S_M,             // values in the current T stream (k or len)
        S_NB,            // its blocks
        S_T0 = 15,       // slot 0 only: the warp's start time in 2^20-cycle units
        S_ROOT = 16,     // W words: the message of the current layer
        S_KEY = 24,      // 8 words: SHA-256 midstate of PUB_SEED, or PUB_SEED itself (SHAKE)
        S_LENS = 32,     // LEN bytes (17 words)
        S_MASK = 49,     // 3 words: bit c set when chain c's end value is in the stream
        S_HDR = 52,      // stream starts here (16-byte aligned)
    };
    enum : uint32_t { EMPTY = 0, ACTIVE = 1, ADVANCE = 2, DEAD = 3 };
    enum : int { K_NONE = 0, K_CHAIN = 1, K_T = 2, K_ROOT = 3 };

    // last value index that block j of a T stream over m values reads
    SPX_DEV static int block_last_value(int j, int m) {
        const int hi = BLK * (j + 1) - 1 - PRE;
        const int last = hi < 0 ? -1 : hi / N;
        return last < m - 1 ? last : m - 1;
    }
    // number of leading finished chains (first clear bit of the 96-bit mask)
    SPX_DEV static int done_prefix(const uint32_t *S) {
        const uint32_t a = S[S_MASK], b = S[S_MASK + 1], c = S[S_MASK + 2];
        if (~a) return __ffs(~a) - 1;
        if (~b) return 32 + __ffs(~b) - 1;
        if (~c) return 64 + __ffs(~c) - 1;
        return 96;
    }
    SPX_DEV static void mark_done(uint32_t *S, int c) { atomicOr(&S[S_MASK + (c >> 5)], 1u << (c & 31)); }
    // initial mask word q for m values: bits of values >= m read as done
    static constexpr uint32_t mask_init(int q, int m) {
        return m <= 32 * q ? ~0u : (m >= 32 * (q + 1) ? 0u : ~0u << (m - 32 * q));
    }
};

// ---------------------------------------------------------------------------
// SHA-256: stream = ADRS_c (22 B) || values || SHA-256 padding, after the
// PUB_SEED midstate; unit = one compression.  Values sit at offset 22 + c n
// (2 mod 4), so they are read and written with byte permutes.
// ---------------------------------------------------------------------------
template <class HF>
struct VerifySha2 : VerifySlot<4 * HF::W, 22, 64> {
    using B = VerifySlot<4 * HF::W, 22, 64>;
    static constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    static constexpr int stream_blocks(int m) { return (22 + m * N + 9 + 63) / 64; }
    static constexpr int kStreamWords = stream_blocks(LEN) * 16;
    static constexpr int kHBlocks = (22 + 2 * N + 9 + 63) / 64;   // H = SHA256(mid; ADRS_c || l || r)
    // units per F step and per H; whether T absorbs a mask stream
    static constexpr int kFUnits = 1, kHUnits = kHBlocks;
    static constexpr bool kTMask = false;
    static __host__ __device__ int slot_words(int hp) { return B::S_HDR + kStreamWords + hp * W; }

    struct Unit {
        uint32_t st[8], blk[16], out[8];
    };
    struct LaneRegs {
        uint32_t kmid[8];   // the task's key midstate
        uint32_t tst[8];    // T running state / first-block state of a two-block H
    };

    SPX_DEV static void put16(uint32_t *base, int byte_off, uint32_t v) {
        reinterpret_cast<uint16_t *>(base)[byte_off >> 1] = (uint16_t)v;
    }
    // value c (big-endian words) at stream byte 22 + c n
    SPX_DEV static void write_value(uint32_t *stream, int c, const uint32_t v[W]) {
        const int off = 22 + c * N;
        put16(stream, off, __byte_perm(v[0], 0, 0x0023));
#pragma unroll
        for (int i = 0; i + 1 < W; i++) stream[(off + 2) / 4 + i] = __byte_perm(v[i], v[i + 1], 0x6701);
        put16(stream, off + N - 2, __byte_perm(v[W - 1], 0, 0x0001));
    }
    SPX_DEV static void read_value(const uint32_t *stream, int c, uint32_t v[W]) {
        const int w0 = (20 + c * N) / 4;
#pragma unroll
        for (int i = 0; i < W; i++) v[i] = __byte_perm(stream[w0 + i], stream[w0 + i + 1], 0x2345);
    }
    // value bytes 8q .. 8q+7 (memory order) to stream byte 22 + 8q
    SPX_DEV static void put_value_word(uint32_t *stream, int q, uint2 x) {
        const int o = 22 + 8 * q;
        put16(stream, o, x.x);
        stream[(o + 2) / 4] = __byte_perm(x.x, x.y, 0x5432);
        put16(stream, o + 6, x.y >> 16);
    }
    // `bytes` (multiple of 8) from 8-byte aligned global memory to stream
    // byte 22 onwards, warp-cooperatively
    SPX_DEV static void copy_values(uint32_t *stream, const uint8_t *src, int bytes, uint32_t lane) {
        for (int q = lane; q < bytes / 8; q += 32) put_value_word(stream, q, reinterpret_cast<const uint2 *>(src)[q]);
    }
    // ADRS_c prefix and the padding after m values (the length counts the
    // 64-byte midstate block)
    SPX_DEV static void frame(uint32_t *stream, const uint32_t *, const Adrs &a, int m, uint32_t lane) {
        const int end = 22 + m * N;   // = 2 (mod 4)
        const int nb = stream_blocks(m);
        if (lane < 5) stream[lane] = __byte_perm(a.w[lane], 0, 0x0123);
        if (lane == 5) put16(stream, 20, __byte_perm(a.w[5], 0, 0x0023));
        if (lane == 6) put16(stream, end, 0x80u);
        for (int q = (end + 2) / 4 + (int)lane; q < nb * 16 - 2; q += 32) stream[q] = 0;
        if (lane == 7) {
            const uint64_t bits = (uint64_t)(64 + end) * 8;
            stream[nb * 16 - 2] = __byte_perm((uint32_t)(bits >> 32), 0, 0x0123);
            stream[nb * 16 - 1] = __byte_perm((uint32_t)bits, 0, 0x0123);
        }
    }
    SPX_DEV static void load_key(uint32_t *S, const SignWork *wk, const uint8_t *, uint32_t lane) {
        if (lane < 8) S[B::S_KEY + lane] = wk->mid[lane];
    }

    SPX_DEV static void claim_chain(LaneRegs &r, const uint32_t *S) {
#pragma unroll
        for (int i = 0; i < 8; i++) r.kmid[i] = S[B::S_KEY + i];
    }
    SPX_DEV static void claim_t(LaneRegs &r, uint32_t *S, int) {
#pragma unroll
        for (int i = 0; i < 8; i++) r.kmid[i] = r.tst[i] = S[B::S_KEY + i];
    }

    SPX_DEV static void build_chain(Unit &u, const LaneRegs &r, const uint32_t *S, int c, int s, int,
                                    const uint32_t v[W]) {
#pragma unroll
        for (int i = 0; i < 8; i++) u.st[i] = r.kmid[i];
        u.blk[0] = S[B::S_AW0];
        u.blk[1] = S[B::S_AW1];
        u.blk[2] = S[B::S_AW2];
        u.blk[3] = S[B::S_IDXL] << 16;
        u.blk[4] = (uint32_t)c << 16;
        u.blk[5] = ((uint32_t)s << 16) | (v[0] >> 16);
#pragma unroll
        for (int i = 1; i < W; i++) u.blk[5 + i] = __funnelshift_l(v[i], v[i - 1], 16);
        u.blk[5 + W] = (v[W - 1] << 16) | 0x8000u;
#pragma unroll
        for (int i = 6 + W; i < 15; i++) u.blk[i] = 0;
        u.blk[15] = (64 + 22 + N) * 8;
    }
    SPX_DEV static void build_t(Unit &u, const LaneRegs &r, uint32_t *S, int j, int) {
        const uint32_t *b = S + B::S_HDR + j * 16;
#pragma unroll
        for (int i = 0; i < 8; i++) u.st[i] = r.tst[i];
#pragma unroll
        for (int i = 0; i < 16; i++) u.blk[i] = __byte_perm(b[i], 0, 0x0123);
    }
    // H of compute_root at height h -> h + 1 for node index idx; sub = block
    SPX_DEV static void build_h(Unit &u, const LaneRegs &r, const uint32_t *S, int h, int sub, uint32_t idx,
                                const uint32_t v[W], int) {
        uint32_t sib[W];
        const uint32_t *auth = S + B::S_HDR + kStreamWords + h * W;
#pragma unroll
        for (int i = 0; i < W; i++) sib[i] = __byte_perm(auth[i], 0, 0x0123);
        const bool right = idx & 1u;
        uint32_t in[2 * W];
#pragma unroll
        for (int i = 0; i < W; i++) {
            in[i] = right ? sib[i] : v[i];
            in[W + i] = right ? v[i] : sib[i];
        }
        Adrs a;
        a.w[0] = S[B::S_AW0];
        a.w[1] = S[B::S_AW1];
        a.w[2] = (S[B::S_AW2] & 0xff000000u) | (ADDR_HASHTREE << 16);
        a.w[3] = 0;
        a.w[4] = 0;
        a.w[5] = 0;
        adrs_height(a, h + 1);
        adrs_index(a, idx >> 1);
        constexpr int TOT = 22 + 2 * N;
        uint32_t m[16 * kHBlocks];
#pragma unroll
        for (int i = 0; i < 5; i++) m[i] = a.w[i];
        m[5] = (a.w[5] & 0xffff0000u) | (in[0] >> 16);
#pragma unroll
        for (int i = 1; i < 2 * W; i++) m[5 + i] = __funnelshift_l(in[i], in[i - 1], 16);
        m[5 + 2 * W] = (in[2 * W - 1] << 16) | 0x8000u;
#pragma unroll
        for (int i = 6 + 2 * W; i < 16 * kHBlocks; i++) m[i] = 0;
        m[16 * kHBlocks - 1] = (64 + TOT) * 8;
        if (kHBlocks == 1 || sub == 0) {
#pragma unroll
            for (int i = 0; i < 8; i++) u.st[i] = r.kmid[i];
#pragma unroll
            for (int i = 0; i < 16; i++) u.blk[i] = m[i];
        } else {
#pragma unroll
            for (int i = 0; i < 8; i++) u.st[i] = r.tst[i];
#pragma unroll
            for (int i = 0; i < 16; i++) u.blk[i] = m[16 * (kHBlocks - 1) + i];
        }
    }
    SPX_DEV static void build_idle(Unit &u) {
#pragma unroll
        for (int i = 0; i < 8; i++) u.st[i] = 0;
#pragma unroll
        for (int i = 0; i < 16; i++) u.blk[i] = 0;
    }
    SPX_DEV static void run(Unit &u) {
#pragma unroll
        for (int i = 0; i < 8; i++) u.out[i] = u.st[i];
        sha256_rounds<0, 64>(u.out, u.blk);
#pragma unroll
        for (int i = 0; i < 8; i++) u.out[i] += u.st[i];
    }
    SPX_DEV static void value_out(const Unit &u, uint32_t v[W]) {
#pragma unroll
        for (int i = 0; i < W; i++) v[i] = u.out[i];
    }
    SPX_DEV static void after_t(const Unit &u, LaneRegs &r, uint32_t *, int) {
#pragma unroll
        for (int i = 0; i < 8; i++) r.tst[i] = u.out[i];
    }
    // first block of a two-block H (the only H unit before the last)
    SPX_DEV static void after_h_unit(const Unit &u, LaneRegs &r, int) {
#pragma unroll
        for (int i = 0; i < 8; i++) r.tst[i] = u.out[i];
    }
};

// ---------------------------------------------------------------------------
// SHAKE-256: stream = PUB_SEED || ADRS (32 B) || values || SHAKE padding,
// 64-bit lanes in memory order (thash_shake256.cu:15-25 absorbs exactly
// this); unit = one Keccak-f[1600] with one 17-lane block absorbed.  F and
// H fit one block for every n; the T sponge state (25 lanes) lives in the
// slot, so only the T lane touches it.
// ---------------------------------------------------------------------------
template <class HF>
struct VerifyShake : VerifySlot<4 * HF::W, 4 * HF::W + 32, 136> {
    using B = VerifySlot<4 * HF::W, 4 * HF::W + 32, 136>;
    static constexpr int W = HF::W, N = 4 * W, NL = N / 8, LEN = 2 * N + 3;
    static constexpr int kPreLanes = NL + 4;
    static constexpr int stream_blocks(int m) { return (8 * kPreLanes + m * N) / 136 + 1; }
    static constexpr int kStreamWords = stream_blocks(LEN) * 34;
    static constexpr int kHBlocks = 1;
    static constexpr int kFUnits = 1, kHUnits = 1;
    static constexpr bool kTMask = false;
    static constexpr int kTStateWords = 50;
    static __host__ __device__ int slot_words(int hp) { return B::S_HDR + kStreamWords + hp * W + kTStateWords; }

    struct Unit {
        uint64_t A[25];
    };
    struct LaneRegs {};

    SPX_DEV static uint64_t *lanes(uint32_t *p) { return reinterpret_cast<uint64_t *>(p); }
    SPX_DEV static const uint64_t *lanes(const uint32_t *p) { return reinterpret_cast<const uint64_t *>(p); }
    SPX_DEV static uint64_t *tstate(uint32_t *S, int hp) { return lanes(S + B::S_HDR + kStreamWords + hp * W); }

    SPX_DEV static void write_value(uint32_t *stream, int c, const uint32_t v[W]) {
        uint32_t *d = stream + 2 * (kPreLanes + c * NL);
#pragma unroll
        for (int i = 0; i < W; i++) d[i] = v[i];
    }
    SPX_DEV static void read_value(const uint32_t *stream, int c, uint32_t v[W]) {
        const uint32_t *s = stream + 2 * (kPreLanes + c * NL);
#pragma unroll
        for (int i = 0; i < W; i++) v[i] = s[i];
    }
    // value bytes 8q .. 8q+7 (memory order) to value lane q
    SPX_DEV static void put_value_word(uint32_t *stream, int q, uint2 x) {
        lanes(stream)[kPreLanes + q] = (uint64_t)x.y << 32 | x.x;
    }
    SPX_DEV static void copy_values(uint32_t *stream, const uint8_t *src, int bytes, uint32_t lane) {
        uint64_t *d = lanes(stream) + kPreLanes;
        for (int q = lane; q < bytes / 8; q += 32) d[q] = reinterpret_cast<const uint64_t *>(src)[q];
    }
    // PUB_SEED and ADRS lanes, then the padding after m values
    SPX_DEV static void frame(uint32_t *stream, const uint32_t *S, const Adrs &a, int m, uint32_t lane) {
        uint64_t *L = lanes(stream);
        uint64_t al[4];
        adrs_lanes(a, al);
        if (lane < (uint32_t)NL) L[lane] = lane_of(S[B::S_KEY + 2 * lane], S[B::S_KEY + 2 * lane + 1]);
        if (lane >= (uint32_t)NL && lane < (uint32_t)kPreLanes) L[lane] = al[lane - NL];
        const int end = kPreLanes + m * NL;   // first lane after the values
        const int last = 17 * stream_blocks(m) - 1;
        for (int q = end + (int)lane; q <= last; q += 32)
            L[q] = (q == end ? 0x1Full : 0ull) ^ (q == last ? 0x8000000000000000ull : 0ull);
    }
    SPX_DEV static void load_key(uint32_t *S, const SignWork *, const uint8_t *pk, uint32_t lane) {
        if (lane < (uint32_t)W) S[B::S_KEY + lane] = reinterpret_cast<const uint32_t *>(pk)[lane];
    }

    SPX_DEV static void claim_chain(LaneRegs &, const uint32_t *) {}
    SPX_DEV static void claim_t(LaneRegs &, uint32_t *S, int hp) {
        uint64_t *T = tstate(S, hp);
#pragma unroll
        for (int i = 0; i < 25; i++) T[i] = 0;
    }

    // PUB_SEED || ADRS (ADRS given as its six big-endian words) into lanes 0..NL+3
    SPX_DEV static void put_prefix(Unit &u, const uint32_t *S, const uint32_t aw[6]) {
#pragma unroll
        for (int i = 0; i < NL; i++) u.A[i] = lane_of(S[B::S_KEY + 2 * i], S[B::S_KEY + 2 * i + 1]);
        u.A[NL] = lane_of(bswap32(aw[0]), bswap32(aw[1]));
        u.A[NL + 1] = lane_of(bswap32(aw[2]), bswap32(aw[3]));
        u.A[NL + 2] = lane_of(bswap32(aw[4]), bswap32(aw[5]));
        u.A[NL + 3] = 0;
    }
    SPX_DEV static void build_chain(Unit &u, const LaneRegs &, const uint32_t *S, int c, int s, int,
                                    const uint32_t v[W]) {
#pragma unroll
        for (int i = 0; i < 25; i++) u.A[i] = 0;
        const uint32_t aw[6] = {S[B::S_AW0], S[B::S_AW1], S[B::S_AW2], S[B::S_IDXL] << 16, (uint32_t)c << 16,
                                (uint32_t)s << 16};
        put_prefix(u, S, aw);
#pragma unroll
        for (int i = 0; i < NL; i++) u.A[kPreLanes + i] = lane_of(v[2 * i], v[2 * i + 1]);
        u.A[kPreLanes + NL] = 0x1Full;
        u.A[16] ^= 0x8000000000000000ull;
    }
    SPX_DEV static void build_t(Unit &u, const LaneRegs &, uint32_t *S, int j, int hp) {
        const uint64_t *T = tstate(S, hp);
        const uint64_t *b = lanes(S + B::S_HDR) + 17 * j;
#pragma unroll
        for (int i = 0; i < 17; i++) u.A[i] = T[i] ^ b[i];
#pragma unroll
        for (int i = 17; i < 25; i++) u.A[i] = T[i];
    }
    SPX_DEV static void build_h(Unit &u, const LaneRegs &, const uint32_t *S, int h, int, uint32_t idx,
                                const uint32_t v[W], int) {
        const uint32_t *auth = S + B::S_HDR + kStreamWords + h * W;
        const bool right = idx & 1u;
        Adrs a;
        a.w[0] = S[B::S_AW0];
        a.w[1] = S[B::S_AW1];
        a.w[2] = (S[B::S_AW2] & 0xff000000u) | (ADDR_HASHTREE << 16);
        a.w[3] = 0;
        a.w[4] = 0;
        a.w[5] = 0;
        adrs_height(a, h + 1);
        adrs_index(a, idx >> 1);
#pragma unroll
        for (int i = 0; i < 25; i++) u.A[i] = 0;
        put_prefix(u, S, a.w);
#pragma unroll
        for (int i = 0; i < NL; i++) {
            const uint64_t sl = lane_of(auth[2 * i], auth[2 * i + 1]);
            const uint64_t vl = lane_of(v[2 * i], v[2 * i + 1]);
            u.A[kPreLanes + i] = right ? sl : vl;
            u.A[kPreLanes + NL + i] = right ? vl : sl;
        }
        u.A[kPreLanes + 2 * NL] ^= 0x1Full;
        u.A[16] ^= 0x8000000000000000ull;
    }
    SPX_DEV static void build_idle(Unit &u) {
#pragma unroll
        for (int i = 0; i < 25; i++) u.A[i] = 0;
    }
    SPX_DEV static void run(Unit &u) { keccak_f1600(u.A); }
    SPX_DEV static void value_out(const Unit &u, uint32_t v[W]) {
#pragma unroll
        for (int i = 0; i < NL; i++) { v[2 * i] = (uint32_t)u.A[i]; v[2 * i + 1] = (uint32_t)(u.A[i] >> 32); }
    }
    SPX_DEV static void after_t(const Unit &u, LaneRegs &, uint32_t *S, int hp) {
        uint64_t *T = tstate(S, hp);
#pragma unroll
        for (int i = 0; i < 25; i++) T[i] = u.A[i];
    }
    SPX_DEV static void after_h_unit(const Unit &, LaneRegs &, int) {}
};

// ---------------------------------------------------------------------------
// SHAKE-256 robust (SPHINCS+ round-3 robust tweakable hash; the reference has
// no robust thash): every F and H input is xored with a mask drawn from
// SHAKE256(PUB_SEED || ADRS), and T_l absorbs its values xored with the
// squeezed stream of SHAKE256(PUB_SEED || ADRS_T).  A chain step or an H is
// two units (the mask permutation, then the hash); the T lane is claimed as
// soon as its layer starts and squeezes the mask stream (one permutation per
// 17 lanes) into the slot while the chains run, then absorbs each T block
// once its chains and its mask lanes are there.
// ---------------------------------------------------------------------------
template <class HF>
struct VerifyShakeRobust : VerifyShake<HF> {
    using S0 = VerifyShake<HF>;
    using B = typename S0::B;
    using Unit = typename S0::Unit;
    static constexpr int W = S0::W, N = S0::N, NL = S0::NL, LEN = S0::LEN, kPreLanes = S0::kPreLanes;
    static constexpr int kStreamWords = S0::kStreamWords;
    static constexpr int kFUnits = 2, kHUnits = 2;
    static constexpr bool kTMask = true;
    enum : int { S_MB = 14 };   // header: mask blocks squeezed so far
    static constexpr int mask_blocks(int m) { return (m * NL + 16) / 17; }
    static constexpr int kMaskLanes = 17 * ((LEN * NL + 16) / 17);
    static __host__ __device__ int slot_words(int hp) { return S0::slot_words(hp) + 50 + 2 * kMaskLanes; }

    struct LaneRegs {
        uint64_t mk[2 * NL];   // the current F or H mask
    };

    SPX_DEV static uint64_t *msponge(uint32_t *S, int hp) { return S0::tstate(S, hp) + 25; }
    SPX_DEV static uint64_t *mlanes(uint32_t *S, int hp) { return S0::tstate(S, hp) + 50; }

    SPX_DEV static void claim_chain(LaneRegs &, const uint32_t *) {}
    SPX_DEV static void claim_t(LaneRegs &, uint32_t *S, int hp) {
        uint64_t *T = S0::tstate(S, hp);
#pragma unroll
        for (int i = 0; i < 25; i++) T[i] = 0;
        S[S_MB] = 0;
    }

    // mask unit: SHAKE256(PUB_SEED || ADRS) with nothing after the ADRS
    SPX_DEV static void mask_unit(Unit &u, const uint32_t *S, const uint32_t aw[6]) {
#pragma unroll
        for (int i = 0; i < 25; i++) u.A[i] = 0;
        S0::put_prefix(u, S, aw);
        u.A[kPreLanes] = 0x1Full;
        u.A[16] ^= 0x8000000000000000ull;
    }
    SPX_DEV static void build_chain(Unit &u, const LaneRegs &r, const uint32_t *S, int c, int s, int sub,
                                    const uint32_t v[W]) {
        const uint32_t aw[6] = {S[B::S_AW0], S[B::S_AW1], S[B::S_AW2], S[B::S_IDXL] << 16, (uint32_t)c << 16,
                                (uint32_t)s << 16};
        mask_unit(u, S, aw);
        if (sub == 1) {
            // the masked value replaces the mask unit's pad lane; the pad
            // byte moves behind it (the 0x80 of lane 16 stays)
#pragma unroll
            for (int i = 0; i < NL; i++) u.A[kPreLanes + i] = lane_of(v[2 * i], v[2 * i + 1]) ^ r.mk[i];
            u.A[kPreLanes + NL] = 0x1Full;
        }
    }
    SPX_DEV static void after_f_unit(const Unit &u, LaneRegs &r, int) {
#pragma unroll
        for (int i = 0; i < NL; i++) r.mk[i] = u.A[i];
    }
    SPX_DEV static void build_h(Unit &u, const LaneRegs &r, const uint32_t *S, int h, int sub, uint32_t idx,
                                const uint32_t v[W], int) {
        const uint32_t *auth = S + B::S_HDR + kStreamWords + h * W;
        const bool right = idx & 1u;
        Adrs a;
        a.w[0] = S[B::S_AW0];
        a.w[1] = S[B::S_AW1];
        a.w[2] = (S[B::S_AW2] & 0xff000000u) | (ADDR_HASHTREE << 16);
        a.w[3] = 0;
        a.w[4] = 0;
        a.w[5] = 0;
        adrs_height(a, h + 1);
        adrs_index(a, idx >> 1);
        mask_unit(u, S, a.w);
        if (sub == 1) {
            // masked l || r replace the mask unit's pad lane; pad behind them
#pragma unroll
            for (int i = 0; i < NL; i++) {
                const uint64_t sl = lane_of(auth[2 * i], auth[2 * i + 1]);
                const uint64_t vl = lane_of(v[2 * i], v[2 * i + 1]);
                u.A[kPreLanes + i] = (right ? sl : vl) ^ r.mk[i];
                u.A[kPreLanes + NL + i] = (right ? vl : sl) ^ r.mk[NL + i];
            }
            u.A[kPreLanes + 2 * NL] ^= 0x1Full;
        }
    }
    SPX_DEV static void after_h_unit(const Unit &u, LaneRegs &r, int) {
#pragma unroll
        for (int i = 0; i < 2 * NL; i++) r.mk[i] = u.A[i];
    }

    // T lane's next unit for block j: 1 = a mask block (needed by block j, or
    // ahead of the chains), 0 = block j, 2 = nothing ready
    SPX_DEV static int t_action(const uint32_t *S, int j) {
        const int m = (int)S[B::S_M];
        const int mb = (int)S[S_MB];
        const int hi = 17 * j + 16 - kPreLanes;   // last value lane of block j
        const int last = hi < m * NL - 1 ? hi : m * NL - 1;
        const int need = last < 0 ? 0 : last / 17 + 1;
        if (mb < need) return 1;
        if (B::done_prefix(S) > B::block_last_value(j, m)) return 0;
        return mb < mask_blocks(m) ? 1 : 2;
    }
    SPX_DEV static void build_mask(Unit &u, uint32_t *S, int hp) {
        if (S[S_MB] == 0) {
            const uint64_t *L = S0::lanes(S + B::S_HDR);   // PUB_SEED || ADRS_T lanes of the stream
#pragma unroll
            for (int i = 0; i < 25; i++) u.A[i] = i < kPreLanes ? L[i < kPreLanes ? i : 0] : 0ull;
            u.A[kPreLanes] = 0x1Full;
            u.A[16] ^= 0x8000000000000000ull;
        } else {
            const uint64_t *M = msponge(S, hp);
#pragma unroll
            for (int i = 0; i < 25; i++) u.A[i] = M[i];
        }
    }
    SPX_DEV static void after_mask(const Unit &u, uint32_t *S, int hp) {
        uint64_t *M = msponge(S, hp);
        uint64_t *ml = mlanes(S, hp) + 17 * S[S_MB];
#pragma unroll
        for (int i = 0; i < 25; i++) M[i] = u.A[i];
#pragma unroll
        for (int i = 0; i < 17; i++) ml[i] = u.A[i];
        S[S_MB] = S[S_MB] + 1;
    }
    SPX_DEV static void after_t(const Unit &u, LaneRegs &, uint32_t *S, int hp) {
        uint64_t *T = S0::tstate(S, hp);
#pragma unroll
        for (int i = 0; i < 25; i++) T[i] = u.A[i];
    }
    // T block j with its value lanes xored with the mask stream
    SPX_DEV static void build_t(Unit &u, const LaneRegs &, uint32_t *S, int j, int hp) {
        const uint64_t *T = S0::tstate(S, hp);
        const uint64_t *b = S0::lanes(S + B::S_HDR) + 17 * j;
        const uint64_t *ml = mlanes(S, hp);
        const int nv = (int)S[B::S_M] * NL;
#pragma unroll
        for (int i = 0; i < 17; i++) {
            const int q = 17 * j + i - kPreLanes;   // value lane index
            u.A[i] = T[i] ^ b[i] ^ ((q >= 0 && q < nv) ? ml[q >= 0 && q < nv ? q : 0] : 0ull);
        }
#pragma unroll
        for (int i = 17; i < 25; i++) u.A[i] = T[i];
    }
};

// ---------------------------------------------------------------------------
// Robust SHA-256: every thash input is xored with MGF1-SHA256(PUB_SEED ||
// ADRS_c) before it is hashed (Sha2::thash).  A mask block is
// SHA256(PUB_SEED || ADRS_c || BE32(ctr)) from the IV -- one compression for
// n <= 24, two for n = 32 (kMB units).  A chain step is kMB mask units, then
// the F unit on the masked value; an H is its ceil(2n / 32) mask blocks, then
// its kHBlocks blocks on the masked l || r.  The T lane is claimed as soon as
// its layer starts and computes the T mask (ceil(m n / 32) blocks) into a
// second stream laid out byte for byte like the value stream and zero outside
// the values, while the chains run; block j of T is absorbed with the mask
// stream xored in once its chains and its mask bytes are there.
// ---------------------------------------------------------------------------
template <class HF>
struct VerifySha2Robust : VerifySha2<HF> {
    using S0 = VerifySha2<HF>;
    using B = typename S0::B;
    using Unit = typename S0::Unit;
    static constexpr int W = S0::W, N = S0::N, LEN = S0::LEN;
    static constexpr int kStreamWords = S0::kStreamWords;
    static constexpr int kHBlocks = S0::kHBlocks;
    static constexpr int kMaxHp = 9;                        // tallest subtree of any set
    static constexpr int kMaskTot = N + 26;                 // PUB_SEED || ADRS_c || BE32(ctr)
    static constexpr int kMB = (kMaskTot + 9 + 63) / 64;    // compressions per mask block
    static constexpr int kHMaskBlocks = (2 * N + 31) / 32;
    static constexpr int kFUnits = kMB + 1, kHUnits = kHMaskBlocks * kMB + kHBlocks;
    static constexpr bool kTMask = true;
    enum : int { S_MB = 14 };                               // header: T mask units done
    // after the auth path (sized for kMaxHp): PUB_SEED (W big-endian words),
    // the first-compression state of a T mask block (n = 32), the mask stream
    static constexpr int kPub = B::S_HDR + kStreamWords + kMaxHp * W;
    static constexpr int kMst = kPub + W;
    static constexpr int kMStream = kMst + 8;
    static __host__ __device__ int slot_words(int) { return kMStream + kStreamWords; }

    struct LaneRegs : S0::LaneRegs {
        uint32_t mk[2 * W];   // the current F or H mask
    };

    SPX_DEV static void load_key(uint32_t *S, const SignWork *wk, const uint8_t *pk, uint32_t lane) {
        S0::load_key(S, wk, pk, lane);
        if (lane < W) S[kPub + lane] = bswap32(reinterpret_cast<const uint32_t *>(pk)[lane]);
    }
    // the value stream's frame, and a zero mask stream
    SPX_DEV static void frame(uint32_t *stream, const uint32_t *S, const Adrs &a, int m, uint32_t lane) {
        S0::frame(stream, S, a, m, lane);
        uint32_t *ms = stream + (kMStream - B::S_HDR);
        for (int q = (int)lane; q < kStreamWords; q += 32) ms[q] = 0;
    }
    SPX_DEV static void claim_t(LaneRegs &r, uint32_t *S, int hp) {
        S0::claim_t(r, S, hp);
        S[S_MB] = 0;
    }

    // unit `part` of mask block `ctr` for ADRS words aw (part > 0 resumes
    // from `prev`, the state after the block's first compression)
    SPX_DEV static void mask_unit(Unit &u, const uint32_t *S, const uint32_t aw[6], uint32_t ctr, int part,
                                  const uint32_t prev[8]) {
        if (part == 0) {
#pragma unroll
            for (int i = 0; i < 8; i++) u.st[i] = sha256_iv_word(i);
#pragma unroll
            for (int i = 0; i < W; i++) u.blk[i] = S[kPub + i];
#pragma unroll
            for (int i = 0; i < 5; i++) u.blk[W + i] = aw[i];
            u.blk[W + 5] = (aw[5] & 0xffff0000u) | (ctr >> 16);
            u.blk[W + 6] = (ctr << 16) | 0x8000u;
#pragma unroll
            for (int i = W + 7; i < 16; i++) u.blk[i] = 0;
            if (kMB == 1) u.blk[15] = kMaskTot * 8;
        } else {
#pragma unroll
            for (int i = 0; i < 8; i++) u.st[i] = prev[i];
#pragma unroll
            for (int i = 0; i < 15; i++) u.blk[i] = 0;
            u.blk[15] = kMaskTot * 8;
        }
    }

    SPX_DEV static void build_chain(Unit &u, const LaneRegs &r, const uint32_t *S, int c, int s, int sub,
                                    const uint32_t v[W]) {
        if (sub < kMB) {
            const uint32_t aw[6] = {S[B::S_AW0], S[B::S_AW1], S[B::S_AW2], S[B::S_IDXL] << 16,
                                    (uint32_t)c << 16, (uint32_t)s << 16};
            mask_unit(u, S, aw, 0, sub, r.tst);
        } else {
            uint32_t x[W];
#pragma unroll
            for (int i = 0; i < W; i++) x[i] = v[i] ^ r.mk[i];
            S0::build_chain(u, r, S, c, s, 0, x);
        }
    }
    SPX_DEV static void after_f_unit(const Unit &u, LaneRegs &r, int sub) {
        if (sub < kMB - 1) {
#pragma unroll
            for (int i = 0; i < 8; i++) r.tst[i] = u.out[i];
        } else {
#pragma unroll
            for (int i = 0; i < W; i++) r.mk[i] = u.out[i];
        }
    }

    // H of compute_root at height h -> h + 1 for node index idx; sub: mask
    // units first, then the H blocks
    SPX_DEV static void build_h(Unit &u, const LaneRegs &r, const uint32_t *S, int h, int sub, uint32_t idx,
                                const uint32_t v[W], int) {
        Adrs a;
        a.w[0] = S[B::S_AW0];
        a.w[1] = S[B::S_AW1];
        a.w[2] = (S[B::S_AW2] & 0xff000000u) | (ADDR_HASHTREE << 16);
        a.w[3] = 0;
        a.w[4] = 0;
        a.w[5] = 0;
        adrs_height(a, h + 1);
        adrs_index(a, idx >> 1);
        constexpr int KM = kHMaskBlocks * kMB;
        if (sub < KM) {
            mask_unit(u, S, a.w, (uint32_t)(sub / kMB), sub % kMB, r.tst);
            return;
        }
        const uint32_t *auth = S + B::S_HDR + kStreamWords + h * W;
        const bool right = idx & 1u;
        uint32_t in[2 * W];
#pragma unroll
        for (int i = 0; i < W; i++) {
            const uint32_t sib = __byte_perm(auth[i], 0, 0x0123);
            in[i] = (right ? sib : v[i]) ^ r.mk[i];
            in[W + i] = (right ? v[i] : sib) ^ r.mk[W + i];
        }
        constexpr int TOT = 22 + 2 * N;
        uint32_t m[16 * kHBlocks];
#pragma unroll
        for (int i = 0; i < 5; i++) m[i] = a.w[i];
        m[5] = (a.w[5] & 0xffff0000u) | (in[0] >> 16);
#pragma unroll
        for (int i = 1; i < 2 * W; i++) m[5 + i] = __funnelshift_l(in[i], in[i - 1], 16);
        m[5 + 2 * W] = (in[2 * W - 1] << 16) | 0x8000u;
#pragma unroll
        for (int i = 6 + 2 * W; i < 16 * kHBlocks; i++) m[i] = 0;
        m[16 * kHBlocks - 1] = (64 + TOT) * 8;
        if (kHBlocks == 1 || sub == KM) {
#pragma unroll
            for (int i = 0; i < 8; i++) u.st[i] = r.kmid[i];
#pragma unroll
            for (int i = 0; i < 16; i++) u.blk[i] = m[i];
        } else {
#pragma unroll
            for (int i = 0; i < 8; i++) u.st[i] = r.tst[i];
#pragma unroll
            for (int i = 0; i < 16; i++) u.blk[i] = m[16 * (kHBlocks - 1) + i];
        }
    }
    SPX_DEV static void after_h_unit(const Unit &u, LaneRegs &r, int sub) {
        constexpr int KM = kHMaskBlocks * kMB;
        if (sub < KM && sub % kMB == kMB - 1) {
            // mask block sub / kMB: mask words 8b .. 8b + 7 (indices kept
            // compile-time so mk stays in registers)
#pragma unroll
            for (int b = 0; b < kHMaskBlocks; b++)
                if (b == sub / kMB) {
#pragma unroll
                    for (int i = 0; i < 8; i++)
                        if (8 * b + i < 2 * W) r.mk[8 * b + i] = u.out[i];
                }
        } else {
            // a mask block's first compression, or the first of two H blocks
#pragma unroll
            for (int i = 0; i < 8; i++) r.tst[i] = u.out[i];
        }
    }

    // T lane's next unit for block j: 1 = a mask unit (needed by block j, or
    // ahead of the chains), 0 = block j, 2 = nothing ready
    SPX_DEV static int t_action(const uint32_t *S, int j) {
        const int m = (int)S[B::S_M];
        const int done = (int)S[S_MB] / kMB;                 // complete mask blocks
        const int hi = 64 * j + 41;                           // last value byte block j reads
        const int last = hi < m * N - 1 ? hi : m * N - 1;
        const int need = last / 32 + 1;
        if (done < need) return 1;
        if (B::done_prefix(S) > B::block_last_value(j, m)) return 0;
        return done < (m * N + 31) / 32 ? 1 : 2;
    }
    SPX_DEV static void build_mask(Unit &u, uint32_t *S, int) {
        const int units = (int)S[S_MB];
        const uint32_t *st = S + B::S_HDR;   // the T ADRS_c, in memory order
        uint32_t aw[6];
#pragma unroll
        for (int i = 0; i < 5; i++) aw[i] = bswap32(st[i]);
        aw[5] = bswap32(st[5]) & 0xffff0000u;
        uint32_t prev[8];
#pragma unroll
        for (int i = 0; i < 8; i++) prev[i] = S[kMst + i];
        mask_unit(u, S, aw, (uint32_t)(units / kMB), units % kMB, prev);
    }
    // `nw` big-endian words at mask-stream byte `off` (2 mod 4), like write_value
    SPX_DEV static void write_mask(uint32_t *base, int off, const uint32_t w[8], int nw) {
        S0::put16(base, off, __byte_perm(w[0], 0, 0x0023));
#pragma unroll
        for (int i = 0; i < 7; i++)
            if (i + 1 < nw) base[(off + 2) / 4 + i] = __byte_perm(w[i], w[i + 1], 0x6701);
        uint32_t lastw = w[0];
#pragma unroll
        for (int i = 1; i < 8; i++)
            if (i == nw - 1) lastw = w[i];
        S0::put16(base, off + 4 * nw - 2, __byte_perm(lastw, 0, 0x0001));
    }
    SPX_DEV static void after_mask(const Unit &u, uint32_t *S, int) {
        const int units = (int)S[S_MB];
        const int b = units / kMB;
        if (units % kMB < kMB - 1) {
#pragma unroll
            for (int i = 0; i < 8; i++) S[kMst + i] = u.out[i];
        } else {
            const int m = (int)S[B::S_M];
            const int left = m * N - 32 * b;                  // mask bytes still to place (> 0)
            write_mask(S + kMStream, 22 + 32 * b, u.out, (left < 32 ? left : 32) / 4);
        }
        S[S_MB] = (uint32_t)(units + 1);
    }
    // T block j with its value bytes xored with the mask stream
    SPX_DEV static void build_t(Unit &u, const LaneRegs &r, uint32_t *S, int j, int) {
        const uint32_t *b = S + B::S_HDR + j * 16;
        const uint32_t *mb = S + kMStream + j * 16;
#pragma unroll
        for (int i = 0; i < 8; i++) u.st[i] = r.tst[i];
#pragma unroll
        for (int i = 0; i < 16; i++) u.blk[i] = __byte_perm(b[i] ^ mb[i], 0, 0x0123);
    }
};

template <class HF>
using VerifyPolicy = typename std::conditional<
    HF::kShake != 0, typename std::conditional<HF::kRobust, VerifyShakeRobust<HF>, VerifyShake<HF>>::type,
    typename std::conditional<HF::kRobust, VerifySha2Robust<HF>, VerifySha2<HF>>::type>::type;

// 20 s at 2 GHz in 2^20-cycle units: far beyond any batch's run time
// (16384 robust SHAKE-256f items take 94 ms)
constexpr uint32_t kHyperLimitUnits = 38147;

template <class HF>
__global__ void __launch_bounds__(128) k_verify_hyper(SetParams P, VerifyArgs A, uint32_t *ctr, int G,
                                                      int claim_min) {
    using PV = VerifyPolicy<HF>;
    constexpr int W = PV::W, N = PV::N, LEN = PV::LEN;
    extern __shared__ uint32_t smem[];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int SW = PV::slot_words(P.hp);
    uint32_t *slots = smem + (threadIdx.x >> 5) * G * SW;

    for (int g = lane; g < G; g += 32) slots[g * SW + PV::S_STATE] = PV::EMPTY;
    __syncwarp();

    // lane task state
    int kind = PV::K_NONE, tg = 0;   // task kind, slot
    int tc = 0;                      // chain index / T block / H step
    int ts = 0;                      // chain step / H unit
    int tsub = 0;                    // unit within a chain step (robust: mask, then F)
    int tact = 0;                    // T lane's unit this iteration (robust: 0 block, 1 mask, 2 none)
    uint32_t tidx = 0;               // compute_root node index
    uint32_t v[W];                   // chain value / current node
#pragma unroll
    for (int i = 0; i < W; i++) v[i] = 0;
    typename PV::LaneRegs lr{};
    bool upkeep = true;   // a slot may be empty or waiting for its next layer
    // warp-uniform: slots that may still have a chain or the T stream to hand
    // out, so the claim loop reads nothing for the others (SHA-256-128f at
    // 4096 items -2.3%, robust SHAKE-256f -8%)
    uint32_t open = 0;
    // warp-uniform: slots whose T stream has no lane yet (the critical path:
    // always claimed at once); chains are handed out only once at least
    // claim_min lanes are free, so the claim pass runs less often
    uint32_t tpend = 0;
    // safety net: a warp that has run longer than kHyperCycleLimit clock
    // cycles gives up, marking its unfinished items -3 (the loop always
    // progresses; this bounds it even so).  The start time lives in slot 0's
    // header, in 2^20-cycle units, so it holds no register.
    if (lane == 0) slots[PV::S_T0] = (uint32_t)(clock64() >> 20);
    __syncwarp();

    while (true) {
        if (__any_sync(0xffffffffu, (uint32_t)(clock64() >> 20) - slots[PV::S_T0] > kHyperLimitUnits)) {
            for (int g = 0; g < G; g++) {
                const uint32_t *S = slots + g * SW;
                const uint32_t st = S[PV::S_STATE];
                if (lane == 0 && (st == PV::ACTIVE || st == PV::ADVANCE)) A.verdict[S[PV::S_ITEM]] = -3;
            }
            while (true) {   // and every item not taken yet
                uint32_t it = 0;
                if (lane == 0) it = atomicAdd(ctr, 1u);
                it = __shfl_sync(0xffffffffu, it, 0);
                if (it >= A.count) break;
                if (lane == 0) A.verdict[it] = -3;
            }
            break;
        }
        // ---- slot upkeep: refill empty slots, set up layers (warp-uniform) ----
        for (int g = 0; upkeep && g < G; g++) {
            uint32_t *S = slots + g * SW;
            uint32_t *stream = S + PV::S_HDR;
            while (S[PV::S_STATE] == PV::EMPTY) {
                uint32_t it = 0;
                if (lane == 0) it = atomicAdd(ctr, 1u);
                it = __shfl_sync(0xffffffffu, it, 0);
                if (it >= A.count) {
                    __syncwarp();
                    if (lane == 0) S[PV::S_STATE] = PV::DEAD;
                    __syncwarp();
                    break;
                }
                const SignWork *wk = A.work + it;
                const uint32_t flags = wk->flags;
                if (flags) {
                    if (lane == 0) A.verdict[it] = -1;   // wrong signature length
                    continue;
                }
                const uint64_t tree = wk->tree;
                const uint32_t idx_leaf = wk->idx_leaf;
                PV::load_key(S, wk, A.pk.row(it), lane);
                // T_k over the FORS roots (fors.cu:141-142)
                Adrs pa;
                adrs_zero(pa);
                adrs_tree(pa, tree);
                adrs_keypair(pa, idx_leaf);
                adrs_type(pa, ADDR_FORSPK);
                __syncwarp();
                PV::frame(stream, S, pa, P.k, lane);
                PV::copy_values(stream, A.fors_roots + (uint64_t)it * P.k * N, P.k * N, lane);
                __syncwarp();
                if (lane == 0) {
                    S[PV::S_ITEM] = it;
                    S[PV::S_LAYER] = (uint32_t)-1;
                    S[PV::S_NEXT] = LEN;
                    S[PV::S_TCLAIM] = 0;
                    S[PV::S_TREE_LO] = (uint32_t)tree;
                    S[PV::S_TREE_HI] = (uint32_t)(tree >> 32);
                    S[PV::S_IDX_LEAF] = idx_leaf;
                    S[PV::S_M] = P.k;
                    S[PV::S_NB] = PV::stream_blocks(P.k);
                    S[PV::S_MASK] = S[PV::S_MASK + 1] = S[PV::S_MASK + 2] = ~0u;   // all roots present
                    S[PV::S_STATE] = PV::ACTIVE;
                }
                open |= 1u << g;
                tpend |= 1u << g;
                __syncwarp();
            }
            if (S[PV::S_STATE] == PV::ADVANCE) {
                const int L = (int)S[PV::S_LAYER] + 1;
                const uint32_t it = S[PV::S_ITEM];
                const uint64_t tree = ((uint64_t)S[PV::S_TREE_HI] << 32) | S[PV::S_TREE_LO];
                uint64_t tree_L;
                uint32_t idx_L;
                layer_index(P, tree, S[PV::S_IDX_LEAF], L, tree_L, idx_L);
                uint32_t root[W];
#pragma unroll
                for (int i = 0; i < W; i++) root[i] = S[PV::S_ROOT + i];
                uint8_t *lens = reinterpret_cast<uint8_t *>(S + PV::S_LENS);
                for (int c = lane; c < LEN; c += 32) lens[c] = (uint8_t)chain_len<HF>(P, root, c);
                Adrs pa;
                adrs_zero(pa);
                adrs_layer(pa, L);
                adrs_tree(pa, tree_L);
                adrs_keypair(pa, idx_L);
                adrs_type(pa, ADDR_WOTSPK);
                PV::frame(stream, S, pa, LEN, lane);
                const uint8_t *sl = A.sig + (uint64_t)it * A.sig_stride + N + P.fors_bytes +
                                    (uint64_t)L * (P.wots_bytes + P.hp * N);
                PV::copy_values(stream, sl, LEN * N, lane);
                uint32_t *auth = stream + PV::kStreamWords;
                for (int q = lane; q < P.hp * W; q += 32)
                    auth[q] = reinterpret_cast<const uint32_t *>(sl + P.wots_bytes)[q];
                __syncwarp();
                if (lane == 0) {
                    Adrs wa;   // chain address without chain and hash fields
                    adrs_zero(wa);
                    adrs_layer(wa, L);
                    adrs_tree(wa, tree_L);
                    adrs_type(wa, ADDR_WOTS);
                    adrs_keypair(wa, idx_L);
                    S[PV::S_AW0] = wa.w[0];
                    S[PV::S_AW1] = wa.w[1];
                    S[PV::S_AW2] = wa.w[2];
                    S[PV::S_IDXL] = idx_L;
                    S[PV::S_LAYER] = (uint32_t)L;
                    S[PV::S_NEXT] = 0;
                    S[PV::S_TCLAIM] = 0;
                    S[PV::S_M] = LEN;
                    S[PV::S_NB] = PV::stream_blocks(LEN);
                    S[PV::S_MASK] = PV::mask_init(0, LEN);
                    S[PV::S_MASK + 1] = PV::mask_init(1, LEN);
                    S[PV::S_MASK + 2] = PV::mask_init(2, LEN);
                    S[PV::S_STATE] = PV::ACTIVE;
                }
                open |= 1u << g;
                tpend |= 1u << g;
                __syncwarp();
            }
        }
        upkeep = false;

        // ---- task claims (warp-uniform; slot order is priority order, and
        // within a slot the T stream -- the critical path -- comes first) ----
        uint32_t need = __ballot_sync(0xffffffffu, kind == PV::K_NONE);
        // Chains are also handed out whenever no lane holds a chain or an
        // auth-path task: the busy lanes are then T streams, which may be
        // waiting for exactly those chains, so holding them back could stall
        // the warp for good.  Chain and auth-path tasks always finish within
        // a bounded number of units, so claims are never postponed for long.
        const bool chain_claims = __popc(need) >= claim_min ||
                                  !__any_sync(0xffffffffu, kind == PV::K_CHAIN || kind == PV::K_ROOT);
        for (uint32_t om = open & (chain_claims ? ~0u : tpend); om && need; om &= om - 1) {
            const int g = __ffs(om) - 1;
            uint32_t *S = slots + g * SW;
            if (S[PV::S_STATE] != PV::ACTIVE) {
                open &= ~(1u << g);   // the upkeep sets it again
                continue;
            }
            // (a masked T starts at once: its mask stream needs no chain)
            if (S[PV::S_TCLAIM] == 0 &&
                (PV::kTMask || PV::done_prefix(S) > PV::block_last_value(0, (int)S[PV::S_M]))) {
                const int leader = __ffs(need) - 1;
                if ((int)lane == leader) {
                    kind = PV::K_T;
                    tg = g;
                    tc = 0;
                    PV::claim_t(lr, S, P.hp);
                }
                __syncwarp();
                if (lane == 0) S[PV::S_TCLAIM] = 1;
                tpend &= ~(1u << g);
                __syncwarp();
                need &= ~(1u << leader);
            }
            const uint8_t *lens = reinterpret_cast<const uint8_t *>(S + PV::S_LENS);
            while (need && chain_claims) {
                const int next = (int)S[PV::S_NEXT];
                if (next >= LEN) break;
                const int rank = __popc(need & lt_mask);
                const bool mine = ((need >> lane) & 1u) && next + rank < LEN;
                if (mine) {
                    const int c = next + rank;
                    const int s0 = lens[c];
                    if (s0 >= 15) {
                        PV::mark_done(S, c);   // the signature value is the chain end, already in place
                    } else {
                        kind = PV::K_CHAIN;
                        tg = g;
                        tc = c;
                        ts = s0;
                        tsub = 0;
                        PV::read_value(S + PV::S_HDR, c, v);
                        PV::claim_chain(lr, S);
                    }
                }
                const int taken = min(__popc(need), LEN - next);
                __syncwarp();
                if (lane == 0) S[PV::S_NEXT] = next + taken;
                __syncwarp();
                need = __ballot_sync(0xffffffffu, kind == PV::K_NONE);
            }
            // lanes still free: every chain of the slot is handed out; with
            // the T stream taken too there is nothing more until the slot's
            // next layer (set again by the upkeep)
            if (chain_claims && need && S[PV::S_TCLAIM] != 0) open &= ~(1u << g);
        }
        if (!__any_sync(0xffffffffu, kind != PV::K_NONE)) break;

        // ---- build this lane's unit of the hash ----
        uint32_t *S = slots + tg * SW;
        bool run = kind != PV::K_NONE;
        typename PV::Unit u;
        if (kind == PV::K_CHAIN) {
            PV::build_chain(u, lr, S, tc, ts, tsub, v);
        } else if (kind == PV::K_T) {
            if constexpr (PV::kTMask) {
                tact = PV::t_action(S, tc);
                run = tact != 2;
                if (tact == 1) PV::build_mask(u, S, P.hp);
                else PV::build_t(u, lr, S, tc, P.hp);
            } else {
                // idle while the chains this block covers are still running
                run = PV::done_prefix(S) > PV::block_last_value(tc, (int)S[PV::S_M]);
                PV::build_t(u, lr, S, tc, P.hp);
            }
        } else if (kind == PV::K_ROOT) {
            PV::build_h(u, lr, S, tc, ts, tidx, v, P.hp);
        } else {
            PV::build_idle(u);
        }

        // ---- one unit of the hash, converged across the warp ----
        PV::run(u);

        // ---- use the output ----
        bool slot_event = false;
        bool step = true;   // the chain step's last unit ran
        if constexpr (PV::kFUnits > 1) {
            if (run && kind == PV::K_CHAIN) {
                step = tsub == PV::kFUnits - 1;
                if (!step) PV::after_f_unit(u, lr, tsub);
                tsub = step ? 0 : tsub + 1;
            }
        }
        if constexpr (PV::kTMask) {
            if (run && kind == PV::K_T && tact == 1) {
                PV::after_mask(u, S, P.hp);
                run = false;   // a mask unit does not advance the T stream
            }
        }
        if (run && step && kind == PV::K_CHAIN) {
            PV::value_out(u, v);
            if (++ts >= 15) {
                // the T lane reads this value only after the __syncwarp that
                // ends the iteration (slots are warp-private), so no fence
                PV::write_value(S + PV::S_HDR, tc, v);
                PV::mark_done(S, tc);
                kind = PV::K_NONE;
            }
        } else if (run && kind == PV::K_T) {
            PV::after_t(u, lr, S, P.hp);
            if (++tc >= (int)S[PV::S_NB]) {
                PV::value_out(u, v);
                if ((int)S[PV::S_LAYER] < 0) {
                    // FORS public key: the message of layer 0
#pragma unroll
                    for (int i = 0; i < W; i++) S[PV::S_ROOT + i] = v[i];
                    S[PV::S_STATE] = PV::ADVANCE;
                    slot_event = true;
                    kind = PV::K_NONE;
                } else {
                    kind = PV::K_ROOT;   // leaf done: climb the auth path
                    tc = 0;
                    ts = 0;
                    tidx = S[PV::S_IDXL];
                }
            }
        } else if (run && kind == PV::K_ROOT) {
            if (ts < PV::kHUnits - 1) {
                PV::after_h_unit(u, lr, ts);
                ts++;
            } else {
                PV::value_out(u, v);
                ts = 0;
                tidx >>= 1;
                if (++tc >= P.hp) {
                    const int L = (int)S[PV::S_LAYER];
                    if (L == P.d - 1) {
                        const uint32_t it = S[PV::S_ITEM];
                        uint32_t pr[W];
                        HF::load(pr, A.pk.row(it) + N);
                        bool ok = true;
#pragma unroll
                        for (int i = 0; i < W; i++) ok &= pr[i] == v[i];
                        A.verdict[it] = ok ? 0 : -1;
                        S[PV::S_STATE] = PV::EMPTY;
                    } else {
#pragma unroll
                        for (int i = 0; i < W; i++) S[PV::S_ROOT + i] = v[i];
                        S[PV::S_STATE] = PV::ADVANCE;
                    }
                    slot_event = true;
                    kind = PV::K_NONE;
                }
            }
        }
        upkeep = __any_sync(0xffffffffu, slot_event);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Per-item verify for small batches (crypto_sign_verify, sign.cu:3048-3121).
//
// A lone item is bound by its serial path: per layer the longest WOTS+ chain
// (up to 15 F), the T_len blocks after it and h' H.  Here one block holds
// one item in a single slot of the persistent kernel's layout: thread c of
// the ceil(len / 32) chain warps runs chain c of every layer with the chain
// step precompute (f_prepare / f_step: rounds 0-4 of each SHA-256 F are
// shared by the whole chain), writes the chain end into the slot's T stream
// and sets its done bit; lane 0 of the last warp (the T warp) absorbs each
// T block as soon as the chains it covers are done, then climbs the auth
// path, and the T warp frames the next layer's stream.  One __syncthreads
// per layer hands the root to the chain threads.  What a layer needs that
// does not depend on the root of the layer below -- each chain's signature
// value and step precompute, the auth path -- is fetched during the
// previous layer, off the critical path.  The chain threads never
// wait; the T lane's wait for done bits is bounded (kItemSpinLimit polls,
// each after a short sleep): if it ever ran out the item's verdict is -3
// and the layer loop ends at once.
// ---------------------------------------------------------------------------
constexpr uint32_t kItemSpinLimit = 1u << 22;

template <class HF>
__global__ void __launch_bounds__(128) k_verify_item(SetParams P, VerifyArgs A) {
    using PV = VerifyPolicy<HF>;
    constexpr int W = PV::W, N = PV::N, LEN = PV::LEN;
    constexpr int CW = (LEN + 31) / 32;   // chain warps; warp CW is the T warp
    extern __shared__ uint32_t smem[];
    __shared__ int s_fail;
    uint32_t *S = smem;
    uint32_t *stream = S + PV::S_HDR;
    uint32_t *pre_auth = smem + PV::slot_words(P.hp);   // next layer's auth path (h' x W words)
    const uint32_t tid = threadIdx.x, lane = tid & 31;
    const bool tw = (tid >> 5) == (uint32_t)CW;
    const uint32_t it = blockIdx.x;
    if (it >= A.count) return;   // uniform over the block
    const SignWork *wk = A.work + it;
    if (wk->flags) {   // wrong signature length (sign.cu:3063-3065)
        if (tid == 0) A.verdict[it] = -1;
        return;
    }
    const uint64_t tree = wk->tree;
    const uint32_t idx_leaf = wk->idx_leaf;
    const uint8_t *pk = A.pk.row(it);
    const uint8_t *sig = A.sig + (uint64_t)it * A.sig_stride + N + P.fors_bytes;
    typename PV::LaneRegs lr{};

    // T warp: frame the stream of layer L (ADRS, padding, no value present)
    auto frame_layer = [&](int L) {
        uint64_t tree_L;
        uint32_t idx_L;
        layer_index(P, tree, idx_leaf, L, tree_L, idx_L);
        Adrs pa;
        adrs_zero(pa);
        adrs_layer(pa, L);
        adrs_tree(pa, tree_L);
        adrs_keypair(pa, idx_L);
        adrs_type(pa, ADDR_WOTSPK);
        PV::frame(stream, S, pa, LEN, lane);
        if (lane == 0) {
            Adrs wa;
            adrs_zero(wa);
            adrs_layer(wa, L);
            adrs_tree(wa, tree_L);
            adrs_type(wa, ADDR_WOTS);
            adrs_keypair(wa, idx_L);
            S[PV::S_AW0] = wa.w[0];
            S[PV::S_AW1] = wa.w[1];
            S[PV::S_AW2] = wa.w[2];
            S[PV::S_IDXL] = idx_L;
            S[PV::S_LAYER] = (uint32_t)L;
            S[PV::S_M] = LEN;
            S[PV::S_NB] = PV::stream_blocks(LEN);
            S[PV::S_MASK] = PV::mask_init(0, LEN);
            S[PV::S_MASK + 1] = PV::mask_init(1, LEN);
            S[PV::S_MASK + 2] = PV::mask_init(2, LEN);
        }
        // the auth path of layer L, prefetched into pre_auth
        uint32_t *auth = stream + PV::kStreamWords;
        for (int q = lane; q < P.hp * W; q += 32) auth[q] = pre_auth[q];
    };
    // T warp lanes: the auth path of layer L into pre_auth
    auto fetch_auth = [&](int L, uint32_t from_lane) {
        const uint8_t *sl = sig + (uint64_t)L * (P.wots_bytes + P.hp * N) + P.wots_bytes;
        for (int q = (int)(lane - from_lane); q >= 0 && q < P.hp * W; q += 32 - from_lane)
            pre_auth[q] = reinterpret_cast<const uint32_t *>(sl)[q];
    };
    // T lane: absorb the slot's stream block by block as its values arrive;
    // false if the wait ran out
    auto run_t = [&](uint32_t out[W]) -> bool {
        PV::claim_t(lr, S, P.hp);
        const int nb = (int)S[PV::S_NB];
        const int m = (int)S[PV::S_M];
        uint32_t spins = 0;
        for (int j = 0; j < nb;) {
            int act;
            if constexpr (PV::kTMask) act = PV::t_action(S, j);
            else act = PV::done_prefix(S) > PV::block_last_value(j, m) ? 0 : 2;
            if (act == 2) {
                if (++spins > kItemSpinLimit) return false;
                __nanosleep(64);
                __threadfence_block();   // re-read the done bits; order the value reads after them
                continue;
            }
            __threadfence_block();
            typename PV::Unit u;
            if constexpr (PV::kTMask) {
                if (act == 1) {
                    PV::build_mask(u, S, P.hp);
                    PV::run(u);
                    PV::after_mask(u, S, P.hp);
                    continue;
                }
            }
            PV::build_t(u, lr, S, j, P.hp);
            PV::run(u);
            PV::after_t(u, lr, S, P.hp);
            if (++j == nb) PV::value_out(u, out);
        }
        return true;
    };
    // T lane: root of the current layer's tree from its leaf
    auto climb = [&](uint32_t v[W]) {
        uint32_t idx = S[PV::S_IDXL];
        for (int h = 0; h < P.hp; h++) {
            for (int sub = 0; sub < PV::kHUnits; sub++) {
                typename PV::Unit u;
                PV::build_h(u, lr, S, h, sub, idx, v, P.hp);
                PV::run(u);
                if (sub < PV::kHUnits - 1) PV::after_h_unit(u, lr, sub);
                else PV::value_out(u, v);
            }
            idx >>= 1;
        }
    };

    if (tid == 0) s_fail = 0;
    // ---- T_k over the FORS roots (fors.cu:141-142): the message of layer 0 ----
    if (tw) {
        PV::load_key(S, wk, pk, lane);
        Adrs pa;
        adrs_zero(pa);
        adrs_tree(pa, tree);
        adrs_keypair(pa, idx_leaf);
        adrs_type(pa, ADDR_FORSPK);
        __syncwarp();
        PV::frame(stream, S, pa, P.k, lane);
        PV::copy_values(stream, A.fors_roots + (uint64_t)it * P.k * N, P.k * N, lane);
        if (lane == 0) {
            S[PV::S_LAYER] = (uint32_t)-1;
            S[PV::S_M] = P.k;
            S[PV::S_NB] = PV::stream_blocks(P.k);
            S[PV::S_MASK] = S[PV::S_MASK + 1] = S[PV::S_MASK + 2] = ~0u;   // every value present
        }
        __syncwarp();
        if (lane == 0) {
            uint32_t root[W];
            if (!run_t(root)) s_fail = 1;
#pragma unroll
            for (int i = 0; i < W; i++) S[PV::S_ROOT + i] = root[i];
        } else {
            fetch_auth(0, 1);
        }
        __syncwarp();
        frame_layer(0);
    }
    __syncthreads();

    // ---- the d layers (wots_pk_from_sig + T_len + compute_root each) ----
    KeyRegs<N> key;
    typename HF::FCtx fc;   // chain thread: the step precompute of its chain in the next layer
    uint32_t nv[W];         // and that chain's signature value
    // chain c of layer L: signature value and step precompute (neither
    // depends on the root that sets the chain's length)
    auto fetch_chain = [&](int L, int c) {
        HF::load(nv, sig + (uint64_t)L * (P.wots_bytes + P.hp * N) + (uint64_t)c * N);
        uint64_t tree_L;
        uint32_t idx_L;
        layer_index(P, tree, idx_leaf, L, tree_L, idx_L);
        Adrs wa;
        adrs_zero(wa);
        adrs_layer(wa, L);
        adrs_tree(wa, tree_L);
        adrs_type(wa, ADDR_WOTS);
        adrs_keypair(wa, idx_L);
        adrs_chain(wa, c);
        HF::f_prepare(fc, wa, key);
    };
    if (!tw && tid < LEN) {
        key_from_work<HF>(key, pk, pk, *wk);
        fetch_chain(0, (int)tid);
    }
    for (int L = 0; L < P.d && !s_fail; L++) {
        if (!tw) {
            if (tid < LEN) {
                const int c = (int)tid;
                uint32_t root[W], v[W];
#pragma unroll
                for (int i = 0; i < W; i++) root[i] = S[PV::S_ROOT + i];
                const uint32_t ln = chain_len<HF>(P, root, c);
#pragma unroll
                for (int i = 0; i < W; i++) v[i] = nv[i];
                for (uint32_t s = ln; s < 15; s++) HF::f_step(v, v, fc, s, key);
                PV::write_value(stream, c, v);
                __threadfence_block();   // the value before its done bit
                PV::mark_done(S, c);
                if (L + 1 < P.d) fetch_chain(L + 1, c);
            }
        } else {
            if (lane == 0) {
                uint32_t v[W];
                if (!run_t(v)) {
                    s_fail = 1;
                } else {
                    climb(v);
                    if (L == P.d - 1) {
                        uint32_t pr[W];
                        HF::load(pr, pk + N);
                        bool ok = true;
#pragma unroll
                        for (int i = 0; i < W; i++) ok &= pr[i] == v[i];
                        A.verdict[it] = ok ? 0 : -1;
                    }
#pragma unroll
                    for (int i = 0; i < W; i++) S[PV::S_ROOT + i] = v[i];
                }
            } else if (L + 1 < P.d) {
                fetch_auth(L + 1, 1);   // while lane 0 absorbs T and climbs
            }
            __syncwarp();
            if (L + 1 < P.d && !s_fail) frame_layer(L + 1);
        }
        __syncthreads();
    }
    if (tid == 0 && s_fail) A.verdict[it] = -3;   // a T wait ran out (never expected)
}

}  // namespace cuspx
