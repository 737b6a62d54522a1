// spx_vsort.cuh -- verify kernels that reorganise the WOTS+ chain work:
// layered kernels over each layer's chains sorted by length (large batches,
// this header's first part) and speculative chain runs followed by a serial
// walk (tiny batches, at the end).
//
// crypto_sign_verify (sign.cu:3048-3121) is serial over the d layers of an
// item, and per layer a WOTS+ chain c runs 15 - d_c steps of F
// (wots_pk_from_sig, wots.cu:777-804) where d_c is digit c of the layer's
// message (chain_lengths, wots.cu:84-166): 0 to 15 steps, 7.5 on average.
// A warp that runs 32 chains of mixed lengths side by side is busy for the
// longest of them, so half its lanes idle on average.
//
// Here each layer's chains are bucketed by their number of steps when the
// layer's message becomes known, and the chain kernel hands sorted positions
// to lanes in order: the 32 lanes of a warp hold chains of one length
// (two lengths at a bucket edge), no lane idles and nothing is claimed
// inside the loop.  Buckets are enumerated longest first, so the longest
// chains start in the first blocks the GPU schedules.
//
// Per group of items the launch sequence is
//
//   k_vsort_layer(L = -1)    T_k over the FORS roots; bucket layer 0's chains
//   k_vsort_chains(L = 0)    every chain of layer 0
//   k_vsort_layer(L = 0)     T_len, auth path -> root; bucket layer 1's chains
//   ...
//   k_vsort_layer(L = d-1)   T_len, auth path -> root; compare with PK.root
//
// k_vsort_layer is one thread per item and spends its time in a serial chain
// of ~13 compressions (T_len and the auth path), so the host splits the
// batch into groups on separate streams: one group's layer kernel runs while
// another group's chain kernel keeps the ALU pipes full.
//
// A chain of zero steps is its signature value: it sorts last, and its lane
// in the chain kernel copies the value to the WOTS+ public key buffer.  For
// robust SHA-256 the chain kernel also xors in the value's share of the
// T_len mask (MGF1 blocks are independent), which leaves the layer kernel
// the plain T_len absorb.
#pragma once
#include "spx_verify.cuh"

#define SPX_HD __host__ __device__ __forceinline__

namespace cuspx {

// Chains of each layer bucketed by steps (0..15).  Bucket l holds up to
// `stride` 32-bit entries item << 7 | chain; group g uses entries
// [first_g x len, (first_g + items_g) x len) of every bucket and counters
// cnt[(g x d + L) x 16 + l].
struct VerifyLists {
    uint32_t *tasks = nullptr;   // 16 x stride entries
    uint32_t *cnt = nullptr;     // groups x d x 16 counters, zeroed before the first group starts
    uint64_t stride = 0;         // entries per bucket: at least count x len
    uint8_t *cand = nullptr;     // speculative chain ends: cand_items x d x len x 16 x n, or null
    uint32_t cand_items = 0;
};

// steps of WOTS+ chain c for message msg: 15 - digit c (chain_lengths,
// wots.cu:84-166; w = 16 in every set, so len1 = 2n and len2 = 3); csum is
// the shifted checksum from vsort_checksum.  Called with constant c only
// (unrolled loops), so msg stays in registers.
template <class HF>
SPX_DEV uint32_t vsort_steps(const uint32_t msg[HF::W], uint32_t csum, int c) {
    constexpr int LEN1 = 8 * HF::W, LEN2 = 3;
    uint32_t d;
    if (c < LEN1) {
        uint32_t byte;
        if (HF::kShake) byte = (msg[c >> 3] >> (8 * ((c >> 1) & 3))) & 0xffu;
        else byte = (msg[c >> 3] >> (24 - 8 * ((c >> 1) & 3))) & 0xffu;
        d = (c & 1) ? (byte & 15u) : (byte >> 4);
    } else {
        constexpr int cbits = ((LEN2 * 4 + 7) / 8) * 8;
        d = (csum >> (cbits - 4 * (c - LEN1 + 1))) & 15u;
    }
    return 15u - d;
}
template <class HF>
SPX_DEV uint32_t vsort_checksum(const uint32_t msg[HF::W]) {
    constexpr int LEN1 = 8 * HF::W, LEN2 = 3;
    uint32_t csum = 0;
#pragma unroll
    for (int c = 0; c < LEN1; c++) csum += vsort_steps<HF>(msg, 0, c);
    return csum << ((8 - ((LEN2 * 4) % 8)) % 8);
}

// Robust SHA-256: T_len absorbs its values xored with MGF1 blocks
// SHA256(PUB_SEED || ADRS_T || ctr), which do not depend on one another, so
// the lane that produces chain c's end value xors in the mask words over
// that value (words c W .. c W + W - 1 of the mask stream) and the layer's
// T_len is absorbed without computing the mask stream.  Other sets: no-op.
template <class HF>
SPX_DEV void tlen_mask_value(uint32_t v[HF::W], const KeyRegs<4 * HF::W> &key, int L, uint64_t tree_L,
                             uint32_t idx_L, int c) {
    if constexpr (HF::kRobust && !HF::kShake) {
        constexpr int W = HF::W;
        Adrs ta;
        adrs_zero(ta);
        adrs_layer(ta, L);
        adrs_tree(ta, tree_L);
        adrs_keypair(ta, idx_L);
        adrs_type(ta, ADDR_WOTSPK);
        const uint32_t q0 = (uint32_t)c * W, b0 = q0 >> 3, b1 = (q0 + W - 1) >> 3;
        uint32_t m0[8], m1[8];
        HF::mask_block(m0, key.pub, ta, b0);
        if (b1 != b0) HF::mask_block(m1, key.pub, ta, b1);
#pragma unroll
        for (int i = 0; i < W; i++) {
            const uint32_t q = q0 + i, k = q & 7;
            uint32_t mw = 0;
#pragma unroll
            for (int t = 0; t < 8; t++) mw = (uint32_t)t == k ? ((q >> 3) == b0 ? m0[t] : m1[t]) : mw;
            v[i] ^= mw;
        }
    }
}

// Dynamic shared memory of k_vsort_layer for blocks of b threads: a verify
// slot per thread (spx_verify.cuh: the T input stream in memory byte order,
// the auth path, key material and, for robust sets, the T mask stream), then
// per thread its chains' buckets and ranks for the next layer.
template <class HF>
struct VsortSmem {
    using PV = VerifyPolicy<HF>;
    SPX_HD static uint32_t slot_stride(int hp) { return ((uint32_t)PV::slot_words(hp) + 3u) & ~3u; }
    SPX_HD static uint32_t lr_off(const SetParams &P, uint32_t b) { return b * slot_stride(P.hp) * 4u; }
    SPX_HD static uint32_t bytes(const SetParams &P, uint32_t b) { return lr_off(P, b) + b * (uint32_t)PV::LEN * 4u; }
};

// Root of layer L of one item from its verify slot S, whose stream already
// holds the layer's m values (L = -1: the k FORS roots -> T_k; otherwise the
// len WOTS+ public-key values -> T_len, then compute_root over the auth path
// staged behind the stream).  The item's thread alone writes the slot's key
// material and frame, then runs T and the auth path unit by unit through the
// verify policy (one hash call site per loop, so a warp running alone on its
// SM keeps the code in its instruction cache).  wkp: the item's work record
// in global memory.
template <class HF>
SPX_DEV void vslot_root(const SetParams &P, uint32_t *S, const SignWork &wk, const SignWork *wkp, const uint8_t *pkb,
                        int L, int m, uint32_t root[HF::W]) {
    using PV = VerifyPolicy<HF>;
    constexpr int N = PV::N;
    uint32_t *stream = S + PV::S_HDR;
    // the slot's key material and frame, written by this thread alone
    // (the policy's helpers split them over lanes; all lanes' shares here)
    for (uint32_t l = 0; l < 32; l++) PV::load_key(S, wkp, pkb, l);
    uint64_t tree_L = wk.tree;
    uint32_t idx_L = wk.idx_leaf;
    Adrs pa;
    adrs_zero(pa);
    if (L >= 0) {
        layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
        adrs_layer(pa, L);
    }
    adrs_tree(pa, tree_L);
    adrs_keypair(pa, idx_L);
    adrs_type(pa, L < 0 ? ADDR_FORSPK : ADDR_WOTSPK);
    for (uint32_t l = 0; l < 32; l++) PV::frame(stream, S, pa, m, l);
    Adrs wa;   // the layer's WOTS+ ADRS words, from which build_h derives its own
    adrs_zero(wa);
    adrs_layer(wa, L < 0 ? 0 : L);
    adrs_tree(wa, tree_L);
    adrs_type(wa, ADDR_WOTS);
    adrs_keypair(wa, idx_L);
    S[PV::S_AW0] = wa.w[0];
    S[PV::S_AW1] = wa.w[1];
    S[PV::S_AW2] = wa.w[2];
    S[PV::S_IDXL] = idx_L;
    S[PV::S_M] = (uint32_t)m;
    S[PV::S_NB] = (uint32_t)PV::stream_blocks(m);
    S[PV::S_MASK] = S[PV::S_MASK + 1] = S[PV::S_MASK + 2] = ~0u;   // every value present
    typename PV::LaneRegs lr{};
    PV::claim_t(lr, S, P.hp);
    if constexpr (HF::kRobust && !HF::kShake) {
        // T_len's values arrive masked from the chain kernel: every mask
        // unit reads as done and the slot's mask stream stays zero
        if (L >= 0) S[PV::S_MB] = (uint32_t)(PV::kMB * ((m * N + 31) / 32));
    }
    const int nbk = PV::stream_blocks(m);
    for (int j = 0; j < nbk;) {
        typename PV::Unit u;
        if constexpr (PV::kTMask) {
            if (PV::t_action(S, j) == 1) {
                PV::build_mask(u, S, P.hp);
                PV::run(u);
                PV::after_mask(u, S, P.hp);
                continue;
            }
        }
        PV::build_t(u, lr, S, j, P.hp);
        PV::run(u);
        PV::after_t(u, lr, S, P.hp);
        if (++j == nbk) PV::value_out(u, root);
    }
    if (L >= 0) {
        // compute_root (utils.cu:94-135) over the staged auth path
        uint32_t idx = idx_L;
        for (int h = 0; h < P.hp; h++) {
            for (int sub = 0; sub < PV::kHUnits; sub++) {
                typename PV::Unit u;
                PV::build_h(u, lr, S, h, sub, idx, root, P.hp);
                PV::run(u);
                if (sub < PV::kHUnits - 1) PV::after_h_unit(u, lr, sub);
                else PV::value_out(u, root);
            }
            idx >>= 1;
        }
    }
}

template <class HF>
SPX_DEV void slot_tl(uint32_t *S, const KeyRegs<4 * HF::W> &key, const uint8_t *pub, const Adrs &pa,
                     const uint8_t *vals, int m, uint32_t out[HF::W]) {
    using PV = VerifyPolicy<HF>;
    constexpr int NW = PV::N / 8, kBatch = 16;
    uint32_t *stream = S + PV::S_HDR;
    const uint2 *src = reinterpret_cast<const uint2 *>(vals);
    const int vw = m * NW;
    for (int q0 = 0; q0 < vw; q0 += kBatch) {
        uint2 x[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; k++)
            if (q0 + k < vw) x[k] = src[q0 + k];
#pragma unroll
        for (int k = 0; k < kBatch; k++)
            if (q0 + k < vw) PV::put_value_word(stream, q0 + k, x[k]);
    }
    // key material as the policy lays it out (SHA-256: the PUB_SEED
    // midstate, from a work record; SHAKE and robust SHA-256: PUB_SEED)
    SignWork wk;
#pragma unroll
    for (int i = 0; i < 8; i++) wk.mid[i] = key.mid[i];
    for (uint32_t l = 0; l < 32; l++) PV::load_key(S, &wk, pub, l);
    for (uint32_t l = 0; l < 32; l++) PV::frame(stream, S, pa, m, l);
    S[PV::S_M] = (uint32_t)m;
    S[PV::S_NB] = (uint32_t)PV::stream_blocks(m);
    S[PV::S_MASK] = S[PV::S_MASK + 1] = S[PV::S_MASK + 2] = ~0u;   // every value present
    typename PV::LaneRegs lr{};
    PV::claim_t(lr, S, 0);   // hp 0: no auth path in this slot
    const int nbk = PV::stream_blocks(m);
    for (int j = 0; j < nbk;) {
        typename PV::Unit u;
        if constexpr (PV::kTMask) {
            if (PV::t_action(S, j) == 1) {
                PV::build_mask(u, S, 0);
                PV::run(u);
                PV::after_mask(u, S, 0);
                continue;
            }
        }
        PV::build_t(u, lr, S, j, 0);
        PV::run(u);
        PV::after_t(u, lr, S, 0);
        if (++j == nbk) PV::value_out(u, out);
    }
}

// Thread per item of the group [first, first + n): the root of layer L (T_k
// for L = -1), then either the verdict (L = d-1) or layer L+1's chains
// bucketed by steps.  The block stages its items' values and auth paths into
// their slots with coalesced copies first; each thread then computes its
// item's root (vslot_root).  Dynamic shared memory: VsortSmem<HF>::bytes.
template <class HF>
__global__ void k_vsort_layer(SetParams P, VerifyArgs A, VerifyLists V, int L, uint32_t first, uint32_t n,
                              int grp) {
    using PV = VerifyPolicy<HF>;
    using SM = VsortSmem<HF>;
    constexpr int W = PV::W, N = PV::N, LEN = PV::LEN;
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint32_t hcount[16], hbase[16];
    if (threadIdx.x < 16) hcount[threadIdx.x] = 0;
    const uint32_t stride = SM::slot_stride(P.hp);
    const uint32_t j0 = blockIdx.x * blockDim.x;
    const uint32_t nb = n - j0 < blockDim.x ? n - j0 : blockDim.x;
    const uint32_t i0 = first + j0;
    // the block's values (contiguous over its items) into the slot streams,
    // and its auth paths behind them
    const int m = L < 0 ? P.k : LEN;
    const uint32_t vw = (uint32_t)m * N / 8;
    // (kCopyBatch loads in flight per thread before their stores: one
    // memory latency per batch, not per word; the item and word of a load
    // advance incrementally)
    const uint32_t i = i0 + threadIdx.x;
    const bool live = threadIdx.x < nb;
    SignWork wk;
    wk.flags = 1;
    if (live) wk = A.work[i];
    constexpr int kCopyBatch = 16;
    const uint2 *src = reinterpret_cast<const uint2 *>((L < 0 ? A.fors_roots : A.wpk) + (uint64_t)i0 * m * N);
    {
        uint32_t t = threadIdx.x / vw, q = threadIdx.x - t * vw;
        for (uint32_t w0 = threadIdx.x; w0 < nb * vw; w0 += kCopyBatch * blockDim.x) {
            uint2 x[kCopyBatch];
#pragma unroll
            for (int k = 0; k < kCopyBatch; k++) {
                const uint32_t w = w0 + k * blockDim.x;
                if (w < nb * vw) x[k] = src[w];
            }
#pragma unroll
            for (int k = 0; k < kCopyBatch; k++) {
                if (w0 + k * blockDim.x < nb * vw) PV::put_value_word(smem + t * stride + PV::S_HDR, (int)q, x[k]);
                for (q += blockDim.x; q >= vw; q -= vw) t++;
            }
        }
    }
    if (L >= 0) {
        const uint32_t aw = (uint32_t)P.hp * W;
        const uint8_t *sa = A.sig + (uint64_t)i0 * A.sig_stride + sig_layer_off(P, L) + P.wots_bytes;
        uint32_t t = threadIdx.x / aw, q = threadIdx.x - t * aw;
        for (uint32_t w0 = threadIdx.x; w0 < nb * aw; w0 += kCopyBatch * blockDim.x) {
            uint32_t x[kCopyBatch];
            uint32_t tt = t, qq = q;
#pragma unroll
            for (int k = 0; k < kCopyBatch; k++) {
                if (w0 + k * blockDim.x < nb * aw)
                    x[k] = *reinterpret_cast<const uint32_t *>(sa + (uint64_t)tt * A.sig_stride + 4ull * qq);
                for (qq += blockDim.x; qq >= aw; qq -= aw) tt++;
            }
#pragma unroll
            for (int k = 0; k < kCopyBatch; k++) {
                if (w0 + k * blockDim.x < nb * aw) smem[t * stride + PV::S_HDR + PV::kStreamWords + q] = x[k];
                for (q += blockDim.x; q >= aw; q -= aw) t++;
            }
        }
    }
    __syncthreads();
    const bool ok = live && !wk.flags;
    const uint8_t *pkb = live ? A.pk.row(i) : nullptr;
    uint32_t root[W];
    if (ok) vslot_root<HF>(P, smem + threadIdx.x * stride, wk, A.work + i, pkb, L, m, root);
    if (L == P.d - 1) {   // uniform over the launch: no barrier follows
        if (live) {
            bool eq = ok;
            if (ok) {
                uint32_t pr[W];
                HF::load(pr, pkb + N);
#pragma unroll
                for (int x = 0; x < W; x++) eq &= pr[x] == root[x];
            }
            A.verdict[i] = eq ? 0 : -1;
        }
        return;
    }
    // bucket layer L+1's chains: block-local ranks, one global reservation
    // per bucket and block, then the entries
    uint32_t *lr = reinterpret_cast<uint32_t *>(reinterpret_cast<uint8_t *>(smem) + SM::lr_off(P, blockDim.x)) +
                   threadIdx.x * LEN;
    if (ok) {
        const uint32_t csum = vsort_checksum<HF>(root);
#pragma unroll
        for (int c = 0; c < LEN; c++) {
            const uint32_t l = vsort_steps<HF>(root, csum, c);
            lr[c] = l << 16 | atomicAdd(&hcount[l], 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x < 16 && hcount[threadIdx.x])
        hbase[threadIdx.x] = atomicAdd(&V.cnt[((uint64_t)grp * P.d + L + 1) * 16 + threadIdx.x], hcount[threadIdx.x]);
    __syncthreads();
    if (ok) {
        uint32_t *base = V.tasks + (uint64_t)first * LEN;
        for (int c = 0; c < LEN; c++) {
            const uint32_t e = lr[c], l = e >> 16;
            base[(uint64_t)l * V.stride + hbase[l] + (e & 0xffffu)] = i << 7 | (uint32_t)c;
        }
    }
}

// One lane per chain of layer L, in sorted order (most steps first; the
// zero-step chains, plain copies, last): sorted position p of the group ->
// bucket and entry.
template <class HF>
__global__ void __launch_bounds__(128) k_vsort_chains(SetParams P, VerifyArgs A, VerifyLists V, int L,
                                                      uint32_t first, int grp) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    __shared__ uint32_t cnt[16];
    if (threadIdx.x < 16) cnt[threadIdx.x] = V.cnt[((uint64_t)grp * P.d + L) * 16 + threadIdx.x];
    __syncthreads();
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    int l = 15;
    for (; l >= 0; l--) {
        if (p < cnt[l]) break;
        p -= cnt[l];
    }
    if (l < 0) return;
    const uint32_t e = V.tasks[(uint64_t)first * LEN + (uint64_t)l * V.stride + p];
    const uint32_t item = e >> 7;
    const int c = (int)(e & 127u);
    const SignWork wk = A.work[item];
    const uint8_t *pkb = A.pk.row(item);
    KeyRegs<N> key;
    key_from_work<HF>(key, pkb, pkb, wk);
    uint64_t tree_L;
    uint32_t idx_L;
    layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    Adrs wa;
    adrs_zero(wa);
    adrs_layer(wa, L);
    adrs_tree(wa, tree_L);
    adrs_type(wa, ADDR_WOTS);
    adrs_keypair(wa, idx_L);
    adrs_chain(wa, c);
    typename HF::FCtx fc;
    HF::f_prepare(fc, wa, key);
    uint32_t v[W];
    HF::load(v, A.sig + (uint64_t)item * A.sig_stride + sig_layer_off(P, L) + (uint64_t)c * N);
    for (uint32_t s = 15u - (uint32_t)l; s < 15u; s++) HF::f_step(v, v, fc, s, key);
    tlen_mask_value<HF>(v, key, L, tree_L, idx_L, c);
    HF::store(A.wpk + ((uint64_t)item * LEN + c) * N, v);
}

// ---------------------------------------------------------------------------
// Speculative chains for tiny batches.  A lone item's verify is a serial
// path: per layer the longest WOTS+ chain (up to 15 F), T_len after it and
// the auth path.  The chain lengths of layer L come from layer L-1's root,
// but every chain's start value (its signature value) and its addresses are
// known up front, so k_vspec_cand computes every chain of every layer from
// each of its 16 possible start steps at once, on SMs that a tiny batch
// leaves idle (16 x d x len chain runs per item, 120 F per chain position),
// and k_vspec_walk then walks the layers with T_len and the auth path only,
// taking each chain's end by its digit: ~13 dependent units per layer
// instead of ~20.
// ---------------------------------------------------------------------------

// thread per (start step, item, layer, chain): start-step-major, so a warp's
// lanes run equally many steps
template <class HF>
__global__ void __launch_bounds__(128) k_vspec_cand(SetParams P, VerifyArgs A, uint8_t *cand) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    const uint64_t per_d = (uint64_t)A.count * P.d * LEN;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= 16 * per_d) return;
    const uint32_t dg = (uint32_t)(gid / per_d);
    const uint64_t r = gid - (uint64_t)dg * per_d;
    const uint32_t item = (uint32_t)(r / ((uint64_t)P.d * LEN));
    const uint32_t rem = (uint32_t)(r - (uint64_t)item * P.d * LEN);
    const int L = (int)(rem / LEN), c = (int)(rem - (uint32_t)L * LEN);
    const SignWork wk = A.work[item];
    if (wk.flags) return;
    const uint8_t *pkb = A.pk.row(item);
    KeyRegs<N> key;
    key_from_work<HF>(key, pkb, pkb, wk);
    uint64_t tree_L;
    uint32_t idx_L;
    layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    Adrs wa;
    adrs_zero(wa);
    adrs_layer(wa, L);
    adrs_tree(wa, tree_L);
    adrs_type(wa, ADDR_WOTS);
    adrs_keypair(wa, idx_L);
    adrs_chain(wa, c);
    typename HF::FCtx fc;
    HF::f_prepare(fc, wa, key);
    uint32_t v[W];
    HF::load(v, A.sig + (uint64_t)item * A.sig_stride + sig_layer_off(P, L) + (uint64_t)c * N);
    for (uint32_t st = dg; st < 15u; st++) HF::f_step(v, v, fc, st, key);
    tlen_mask_value<HF>(v, key, L, tree_L, idx_L, c);
    HF::store(cand + ((((uint64_t)item * P.d + L) * LEN + c) * 16 + dg) * N, v);
}

// thread per item: T_k, then per layer the chain ends picked from the
// speculative table by the digits of the layer's message, T_len and the
// auth path (vslot_root); the verdict against PK.root.  Dynamic shared
// memory: blockDim x VsortSmem<HF>::slot_stride words.
template <class HF>
__global__ void __launch_bounds__(32) k_vspec_walk(SetParams P, VerifyArgs A, const uint8_t *cand) {
    using PV = VerifyPolicy<HF>;
    using SM = VsortSmem<HF>;
    constexpr int W = PV::W, N = PV::N, LEN = PV::LEN, NW = N / 8;
    constexpr int kBatch = 24 / NW;   // chain ends loaded before they are stored (24 8-byte words)
    extern __shared__ __align__(16) uint32_t smem[];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.count) return;   // no barriers in this kernel
    const SignWork wk = A.work[i];
    if (wk.flags) {   // wrong signature length (sign.cu:3063-3065)
        A.verdict[i] = -1;
        return;
    }
    const uint8_t *pkb = A.pk.row(i);
    uint32_t *S = smem + threadIdx.x * SM::slot_stride(P.hp);
    uint32_t *stream = S + PV::S_HDR;
    uint32_t root[W];
    {
        const uint2 *src = reinterpret_cast<const uint2 *>(A.fors_roots + (uint64_t)i * P.k * N);
        const int vw = P.k * NW;
        for (int q0 = 0; q0 < vw; q0 += 2 * kBatch) {
            uint2 x[2 * kBatch];
#pragma unroll
            for (int k = 0; k < 2 * kBatch; k++)
                if (q0 + k < vw) x[k] = src[q0 + k];
#pragma unroll
            for (int k = 0; k < 2 * kBatch; k++)
                if (q0 + k < vw) PV::put_value_word(stream, q0 + k, x[k]);
        }
    }
    vslot_root<HF>(P, S, wk, A.work + i, pkb, -1, P.k, root);
    const uint8_t *sig = A.sig + (uint64_t)i * A.sig_stride;
    for (int L = 0; L < P.d; L++) {
        // the layer's auth path behind the stream
        const uint32_t *sa = reinterpret_cast<const uint32_t *>(sig + sig_layer_off(P, L) + P.wots_bytes);
        const int aw = P.hp * W;
        for (int q0 = 0; q0 < aw; q0 += 2 * kBatch) {
            uint32_t x[2 * kBatch];
#pragma unroll
            for (int k = 0; k < 2 * kBatch; k++)
                if (q0 + k < aw) x[k] = sa[q0 + k];
#pragma unroll
            for (int k = 0; k < 2 * kBatch; k++)
                if (q0 + k < aw) S[PV::S_HDR + PV::kStreamWords + q0 + k] = x[k];
        }
        // chain c's end: its run from start step d_c, d_c digit c of the message
        const uint32_t csum = vsort_checksum<HF>(root);
        const uint8_t *cb = cand + ((uint64_t)i * P.d + L) * LEN * 16 * N;
#pragma unroll
        for (int c0 = 0; c0 < LEN; c0 += kBatch) {
            uint2 x[kBatch][NW];
#pragma unroll
            for (int j = 0; j < kBatch; j++) {
                if (c0 + j < LEN) {
                    const uint32_t dg = 15u - vsort_steps<HF>(root, csum, c0 + j);
                    const uint2 *src = reinterpret_cast<const uint2 *>(cb + ((uint64_t)(c0 + j) * 16 + dg) * N);
#pragma unroll
                    for (int h = 0; h < NW; h++) x[j][h] = src[h];
                }
            }
#pragma unroll
            for (int j = 0; j < kBatch; j++)
                if (c0 + j < LEN) {
#pragma unroll
                    for (int h = 0; h < NW; h++) PV::put_value_word(stream, (c0 + j) * NW + h, x[j][h]);
                }
        }
        vslot_root<HF>(P, S, wk, A.work + i, pkb, L, LEN, root);
    }
    uint32_t pr[W];
    HF::load(pr, pkb + N);
    bool eq = true;
#pragma unroll
    for (int x = 0; x < W; x++) eq &= pr[x] == root[x];
    A.verdict[i] = eq ? 0 : -1;
}

}  // namespace cuspx
