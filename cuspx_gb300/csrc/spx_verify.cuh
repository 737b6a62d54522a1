// spx_verify.cuh -- persistent hypertree verify for the SHA-256 simple sets.
//
// crypto_sign_verify (sign.cu:3048-3121) is serial over the d layers of an
// item: layer L's WOTS+ chains (wots_pk_from_sig, wots.cu:777-804) need the
// root of layer L-1, T_len (sign.cu:3103) needs every chain end of layer L,
// and compute_root (utils.cu:94-135) needs T_len.  Per item that is ~10-way
// parallel work on average (35 chains, then one serial T_len + auth path),
// so flat per-layer kernels leave the GPU idle during every T phase.
//
// Here one launch runs the whole hypertree for the batch.  Each warp owns G
// item slots in shared memory and keeps every lane busy with whichever task
// any of its items offers:
//
//   chain   one F per iteration, from the signature value to step 15
//   T       one 64-byte block of T_k (FORS key) or T_len per iteration
//   root    one H compression of compute_root per iteration
//
// T_len streams behind the chains: block j of ADRS_c || ends only needs the
// chains whose end values it covers, so the T lane starts as soon as chains
// 0..2 (n = 16) are done and takes each later block once its chains are; on
// an iteration where its next block is not ready it idles.  This shortens an
// item's per-layer critical path from ~15 + 10 + 3 to ~15 + 2 + 3
// compressions, which is what lets few items per warp keep 32 lanes busy.
//
// Every task is "one SHA-256 compression from a state over a 16-word block";
// lanes differ only in how they build (state, block) and use the output, so
// the compression itself -- the expensive part -- runs converged across the
// warp whatever mix of tasks the lanes hold.  Items are taken from a global
// counter as slots free up, so a batch of any size keeps all warps busy.
//
// Slot data lives in shared memory: the T input stream (ADRS_c || values ||
// padding, memory byte order) into which the layer's WOTS signature is
// copied and where each chain's end value overwrites its start value in
// place, the layer's auth path, the chain lengths, the key midstate and the
// item's position.  Nothing waits on another warp; the loop ends when the
// counter is exhausted and every slot is empty.
#pragma once
#include "spx_kernels.cuh"

namespace cuspx {

template <class HF>
struct PersistVerify {
    static constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    // T stream blocks after the key midstate: ADRS_c (22 B) || m values || pad
    static constexpr int stream_blocks(int m) { return (22 + m * N + 9 + 63) / 64; }
    static constexpr int kStreamWords = stream_blocks(LEN) * 16;
    // H(left, right) = SHA256(midstate; ADRS_c || left || right): blocks
    static constexpr int kHBlocks = (22 + 2 * N + 9 + 63) / 64;

    // slot header word indices
    enum : int {
        S_ITEM = 0, S_LAYER, S_NEXT, S_DONE, S_TCLAIM, S_STATE, S_TREE_LO, S_TREE_HI, S_IDX_LEAF, S_IDXL,
        S_AW0, S_AW1, S_AW2, S_M, S_NB,
        S_ROOT = 16,     // W words
        S_MID = 24,      // 8 words
        S_LENS = 32,     // LEN bytes (17 words)
        S_MASK = 49,     // 3 words: bit c set when chain c's end value is in the stream
        S_HDR = 52,      // stream starts here (16-byte aligned)
    };
    enum : uint32_t { EMPTY = 0, ACTIVE = 1, ADVANCE = 2, DEAD = 3 };
    enum : int { K_NONE = 0, K_CHAIN = 1, K_T = 2, K_ROOT = 3 };

    static __host__ __device__ int slot_words(int hp) { return S_HDR + kStreamWords + hp * W; }

    // last value index that block j of a T stream over m values reads
    SPX_DEV static int block_last_value(int j, int m) {
        const int last = (64 * j + 63 - 22) / N;
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

    // -- byte-stream helpers (stream bytes in memory order, 32-bit words LE) --
    SPX_DEV static void put16(uint32_t *base, int byte_off, uint32_t v) {
        reinterpret_cast<uint16_t *>(base)[byte_off >> 1] = (uint16_t)v;
    }
    // value v (big-endian words) at a stream offset = 2 (mod 4)
    SPX_DEV static void write_value(uint32_t *stream, int off, const uint32_t v[W]) {
        put16(stream, off, __byte_perm(v[0], 0, 0x0023));
#pragma unroll
        for (int i = 0; i + 1 < W; i++) stream[(off + 2) / 4 + i] = __byte_perm(v[i], v[i + 1], 0x6701);
        put16(stream, off + N - 2, __byte_perm(v[W - 1], 0, 0x0001));
    }
    SPX_DEV static void read_value(const uint32_t *stream, int off, uint32_t v[W]) {
        const int w0 = (off - 2) / 4;
#pragma unroll
        for (int i = 0; i < W; i++) v[i] = __byte_perm(stream[w0 + i], stream[w0 + i + 1], 0x2345);
    }
    // copy `bytes` (multiple of 8) from 8-byte aligned global memory to the
    // stream at offset 22, warp-cooperatively
    SPX_DEV static void copy_values(uint32_t *stream, const uint8_t *src, int bytes, uint32_t lane) {
        for (int q = lane; q < bytes / 8; q += 32) {
            const uint2 x = reinterpret_cast<const uint2 *>(src)[q];
            const int o = 22 + 8 * q;
            put16(stream, o, x.x);
            stream[(o + 2) / 4] = __byte_perm(x.x, x.y, 0x5432);
            put16(stream, o + 6, x.y >> 16);
        }
    }
    // ADRS_c prefix (bytes 0..21) and padding after m values, for a T stream
    // over m values: length counts the 64-byte midstate block
    SPX_DEV static void stream_frame(uint32_t *stream, const Adrs &a, int m, uint32_t lane) {
        const int end = 22 + m * N;                 // = 2 (mod 4)
        const int nb = (end + 9 + 63) / 64;
        if (lane < 5) stream[lane] = __byte_perm(a.w[lane], 0, 0x0123);
        if (lane == 5) put16(stream, 20, __byte_perm(a.w[5], 0, 0x0023));
        if (lane == 6) put16(stream, end, 0x80u);
        for (int q = (end + 2) / 4 + lane; q < nb * 16 - 2; q += 32) stream[q] = 0;
        if (lane == 7) {
            const uint64_t bits = (uint64_t)(64 + end) * 8;
            stream[nb * 16 - 2] = __byte_perm((uint32_t)(bits >> 32), 0, 0x0123);
            stream[nb * 16 - 1] = __byte_perm((uint32_t)bits, 0, 0x0123);
        }
    }

    // H block(s): ADRS_c || l || r || pad, total length 64 + 22 + 2n bytes
    SPX_DEV static void h_blocks(uint32_t m[16 * kHBlocks], const Adrs &a, const uint32_t l[W], const uint32_t r[W]) {
        constexpr int TOT = 22 + 2 * N;
        uint32_t in[2 * W];
#pragma unroll
        for (int i = 0; i < W; i++) { in[i] = l[i]; in[W + i] = r[i]; }
#pragma unroll
        for (int i = 0; i < 5; i++) m[i] = a.w[i];
        m[5] = (a.w[5] & 0xffff0000u) | (in[0] >> 16);
#pragma unroll
        for (int i = 1; i < 2 * W; i++) m[5 + i] = __funnelshift_l(in[i], in[i - 1], 16);
        m[5 + 2 * W] = (in[2 * W - 1] << 16) | 0x8000u;
#pragma unroll
        for (int i = 6 + 2 * W; i < 16 * kHBlocks; i++) m[i] = 0;
        m[16 * kHBlocks - 1] = (64 + TOT) * 8;
    }
};

template <class HF>
__global__ void __launch_bounds__(128) k_verify_hyper(SetParams P, VerifyArgs A, uint32_t *ctr, int G) {
    using PV = PersistVerify<HF>;
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
    int ts = 0;                      // chain step / H sub-block
    uint32_t tidx = 0;               // compute_root node index
    uint32_t v[W];                   // chain value / current node
    uint32_t tst[8];                 // T running state / H first-block state
    uint32_t kmid[8];                // the task's key midstate (PUB_SEED block)
#pragma unroll
    for (int i = 0; i < W; i++) v[i] = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) tst[i] = kmid[i] = 0;
    bool upkeep = true;   // a slot may be empty or waiting for its next layer

    while (true) {
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
                if (lane < 8) S[PV::S_MID + lane] = wk->mid[lane];
                // T_k over the FORS roots (fors.cu:141-142)
                Adrs pa;
                adrs_zero(pa);
                adrs_tree(pa, tree);
                adrs_keypair(pa, idx_leaf);
                adrs_type(pa, ADDR_FORSPK);
                __syncwarp();
                PV::stream_frame(stream, pa, P.k, lane);
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
                PV::stream_frame(stream, pa, LEN, lane);
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
                __syncwarp();
            }
        }
        upkeep = false;

        // ---- task claims (warp-uniform; slot order is priority order, and
        // within a slot the T stream -- the critical path -- comes first) ----
        uint32_t need = __ballot_sync(0xffffffffu, kind == PV::K_NONE);
        for (int g = 0; g < G && need; g++) {
            uint32_t *S = slots + g * SW;
            if (S[PV::S_STATE] != PV::ACTIVE) continue;
            if (S[PV::S_TCLAIM] == 0 && PV::done_prefix(S) > PV::block_last_value(0, (int)S[PV::S_M])) {
                const int leader = __ffs(need) - 1;
                if ((int)lane == leader) {
                    kind = PV::K_T;
                    tg = g;
                    tc = 0;
#pragma unroll
                    for (int i = 0; i < 8; i++) kmid[i] = tst[i] = S[PV::S_MID + i];
                }
                __syncwarp();
                if (lane == 0) S[PV::S_TCLAIM] = 1;
                __syncwarp();
                need &= ~(1u << leader);
            }
            const uint8_t *lens = reinterpret_cast<const uint8_t *>(S + PV::S_LENS);
            while (need) {
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
                        PV::read_value(S + PV::S_HDR, 22 + c * N, v);
#pragma unroll
                        for (int i = 0; i < 8; i++) kmid[i] = S[PV::S_MID + i];
                    }
                }
                const int taken = min(__popc(need), LEN - next);
                __syncwarp();
                if (lane == 0) S[PV::S_NEXT] = next + taken;
                __syncwarp();
                need = __ballot_sync(0xffffffffu, kind == PV::K_NONE);
            }
        }
        if (!__any_sync(0xffffffffu, kind != PV::K_NONE)) break;

        // ---- build (state, block) for this lane's compression ----
        uint32_t *S = slots + tg * SW;
        bool run = kind != PV::K_NONE;
        uint32_t st[8], blk[16];
#pragma unroll
        for (int i = 0; i < 8; i++) st[i] = kmid[i];
        if (kind == PV::K_CHAIN) {
            blk[0] = S[PV::S_AW0];
            blk[1] = S[PV::S_AW1];
            blk[2] = S[PV::S_AW2];
            blk[3] = S[PV::S_IDXL] << 16;
            blk[4] = (uint32_t)tc << 16;
            blk[5] = ((uint32_t)ts << 16) | (v[0] >> 16);
#pragma unroll
            for (int i = 1; i < W; i++) blk[5 + i] = __funnelshift_l(v[i], v[i - 1], 16);
            blk[5 + W] = (v[W - 1] << 16) | 0x8000u;
#pragma unroll
            for (int i = 6 + W; i < 15; i++) blk[i] = 0;
            blk[15] = (64 + 22 + N) * 8;
        } else if (kind == PV::K_T) {
            // idle while the chains this block covers are still running
            run = PV::done_prefix(S) > PV::block_last_value(tc, (int)S[PV::S_M]);
            const uint32_t *b = S + PV::S_HDR + tc * 16;
#pragma unroll
            for (int i = 0; i < 8; i++) st[i] = tst[i];
#pragma unroll
            for (int i = 0; i < 16; i++) blk[i] = __byte_perm(b[i], 0, 0x0123);
        } else if (kind == PV::K_ROOT) {
            const int h = tc;   // compute_root step: node at height h -> h + 1
            uint32_t sib[W];
            const uint32_t *auth = S + PV::S_HDR + PV::kStreamWords + h * W;
#pragma unroll
            for (int i = 0; i < W; i++) sib[i] = __byte_perm(auth[i], 0, 0x0123);
            const bool right = tidx & 1u;
            uint32_t l[W], r[W];
#pragma unroll
            for (int i = 0; i < W; i++) {
                l[i] = right ? sib[i] : v[i];
                r[i] = right ? v[i] : sib[i];
            }
            Adrs ta;
            ta.w[0] = S[PV::S_AW0];
            ta.w[1] = S[PV::S_AW1];
            ta.w[2] = (S[PV::S_AW2] & 0xff000000u) | (ADDR_HASHTREE << 16);
            ta.w[3] = 0;
            ta.w[4] = 0;
            ta.w[5] = 0;
            adrs_height(ta, h + 1);
            adrs_index(ta, tidx >> 1);
            uint32_t m[16 * PV::kHBlocks];
            PV::h_blocks(m, ta, l, r);
            if (PV::kHBlocks == 1 || ts == 0) {
#pragma unroll
                for (int i = 0; i < 16; i++) blk[i] = m[i];
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++) st[i] = tst[i];
#pragma unroll
                for (int i = 0; i < 16; i++) blk[i] = m[16 * (PV::kHBlocks - 1) + i];
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; i++) blk[i] = 0;
        }

        // ---- one compression, converged across the warp ----
        uint32_t t[8];
#pragma unroll
        for (int i = 0; i < 8; i++) t[i] = st[i];
        sha256_rounds<0, 64>(t, blk);
#pragma unroll
        for (int i = 0; i < 8; i++) t[i] += st[i];

        // ---- use the output ----
        bool slot_event = false;
        if (run && kind == PV::K_CHAIN) {
#pragma unroll
            for (int i = 0; i < W; i++) v[i] = t[i];
            if (++ts >= 15) {
                PV::write_value(S + PV::S_HDR, 22 + tc * N, v);
                __threadfence_block();   // the end value is in the stream before its done bit
                PV::mark_done(S, tc);
                kind = PV::K_NONE;
            }
        } else if (run && kind == PV::K_T) {
#pragma unroll
            for (int i = 0; i < 8; i++) tst[i] = t[i];
            if (++tc >= (int)S[PV::S_NB]) {
#pragma unroll
                for (int i = 0; i < W; i++) v[i] = t[i];
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
            if (PV::kHBlocks == 2 && ts == 0) {
#pragma unroll
                for (int i = 0; i < 8; i++) tst[i] = t[i];
                ts = 1;
            } else {
#pragma unroll
                for (int i = 0; i < W; i++) v[i] = t[i];
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

}  // namespace cuspx
