// spx_kernels.cuh -- SPHINCS+ keygen / sign / verify kernels, templated on a
// hash family policy (Sha2<N,R> or Shake<N,R>, spx_thash.cuh).
//
// Sign is a fixed pipeline of phase kernels over a batch (captured in a CUDA
// graph by the host engine).  Every phase is flat over independent work so a
// batch of thousands of signatures fills all 152 SMs:
//
//   k_sign_msg      thread / signature   PRF_msg, H_msg -> R, FORS digest, tree, leaf
//   k_sign_msg_wide warp / signature     the same for messages of >= 2 KiB (SHAKE)
//   k_sign_msg_pair 2 warps / 32 sigs    the same for messages of >= 2 KiB (SHA-256):
//                                        schedule warp + rounds warp per message
//   k_fors_sign     2^g lanes / FORS tree leaves (PRF+F), per-lane subtree stack,
//                                        g shuffle levels, auth path, root
//   k_leaves        thread / XMSS leaf   WOTS+ key (len chains x 15 F) streamed into
//                                        T_len; the signing leaf records its chains
//   k_trees         warp / XMSS tree     level-by-level reduction in shared memory,
//                                        auth path, root (k_trees_lane: lane / tree)
//   k_sign_finish   block / signature    FORS pk (T_k), WOTS signatures gathered
//                                        from the recorded chains
//
// Verify: k_verify_msg (+ k_verify_msg_pair / _wide) -> k_verify_fors -> the
// hypertree: for tiny batches every chain run from all 16 start steps, then a
// serial walk (k_vspec_cand + k_vspec_walk, spx_vsort.cuh), one block per
// item for small batches (k_verify_item, spx_verify.cuh), one persistent
// launch for mid-size ones (k_verify_hyper),
// per-layer kernels over length-sorted chains for large ones
// (k_vsort_chains + k_vsort_layer, spx_vsort.cuh); or per-layer
// k_verify_chains + k_verify_root, or k_verify_ht (one thread per item over
// all layers).
// Key generation reuses k_leaves / k_trees on the top layer.
//
// Reference structure followed (CPU form): crypto_sign_signature sign.cu:1924-1994,
// fors_sign fors.cu:107-143, treehash utils.cu:189-241, wots_gen_leaf sign.cu:87-102,
// wots_sign wots.cu:614-625, crypto_sign_verify sign.cu:3048-3121,
// crypto_sign_seed_keypair sign.cu:154-182.
#pragma once
#include "spx_thash.cuh"

namespace cuspx {

// runtime parameter set (params.h:33-146)
struct SetParams {
    int n, h, d, hp, a, k, len, len1, len2;
    int sig_bytes, fors_bytes, wots_bytes, fors_msg_bytes, dgst_bytes;
    int tree_bits, tree_bytes, leaf_bits, leaf_bytes;
    int pk_bytes, sk_bytes;
};

// per-signature plan produced by the message phase (96 bytes): the FORS
// digest, hypertree position and the key's SHA-256 midstate, computed once
// per item instead of once per lane.
struct SignWork {
    uint64_t tree;
    uint32_t idx_leaf;
    uint32_t flags;
    uint8_t mhash[48];
    uint32_t mid[8];
};

// key registers for an item whose midstate is already in its work record
template <class HF>
SPX_DEV void key_from_work(KeyRegs<4 * HF::W> &k, const uint8_t *skseed, const uint8_t *pub, const SignWork &w) {
    HF::load(k.skseed, skseed);
    HF::load(k.pub, pub);
#pragma unroll
    for (int i = 0; i < 8; i++) k.mid[i] = w.mid[i];
}

// Key rows: item i uses key bytes keys + keyrow[i] * key_stride (or row i
// when keyrow is null).  For signing a key row is sk = SK_SEED || SK_PRF ||
// PUB_SEED || ROOT; for verifying it is pk = PUB_SEED || ROOT.
struct KeyRef {
    const uint8_t *keys;
    const uint32_t *keyrow;
    uint32_t stride;
    SPX_DEV const uint8_t *row(uint32_t i) const { return keys + (uint64_t)(keyrow ? keyrow[i] : i) * stride; }
};

struct MsgRef {
    const uint8_t *base;       // 16-byte aligned message slab (slack >= 8 bytes past every message)
    const uint64_t *off;       // per-item byte offset, multiple of 16
    const uint64_t *len;       // per-item length
};

struct SignArgs {
    uint32_t count;
    KeyRef sk;
    MsgRef msg;
    const uint8_t *optrand;    // count x n, or null for the reference's fixed 0xAD.. (sign.cu:1951-1954)
    uint8_t *sig;              // count x sig_bytes
    SignWork *work;            // count
    uint8_t *fors_roots;       // count x k x n
    uint8_t *leaves;           // count x d x 2^hp x n
    uint8_t *roots;            // count x d x n
    uint8_t *chains;           // count x d x len x 16 x n  (signing leaf's chain values)
    int32_t *status;           // count
    uint8_t *ends = nullptr;   // chain-parallel scratch: ends_cap x d x 2^hp x len x n, or null
    uint32_t ends_cap = 0;
};

// tree/leaf indices of hypertree layer L (sign.cu:1987-1988)
SPX_DEV void layer_index(const SetParams &P, uint64_t tree, uint32_t idx_leaf, int L, uint64_t &tree_L,
                         uint32_t &idx_L) {
    const uint32_t mask = (1u << P.hp) - 1u;
    if (L == 0) {
        tree_L = tree;
        idx_L = idx_leaf;
    } else {
        uint64_t t = P.hp * (L - 1) >= 64 ? 0 : (tree >> (P.hp * (L - 1)));
        idx_L = (uint32_t)(t & mask);
        tree_L = P.hp >= 64 ? 0 : (t >> P.hp);
    }
}

// LSB-first FORS index of tree t (message_to_indices, fors.cu:77-88)
SPX_DEV uint32_t fors_index(const uint8_t *mh, int a, int t) {
    uint32_t v = 0;
    int off = t * a;
    for (int j = 0; j < a; j++, off++) v |= ((uint32_t)(mh[off >> 3] >> (off & 7)) & 1u) << j;
    return v;
}

// WOTS+ chain length for chain c of message msg (chain_lengths, wots.cu:84-166):
// base-16 digits MSB nibble first, then the checksum sum(15 - d) shifted left
// by (8 - len2*4 % 8) % 8 and split into len2 digits.
template <class HF>
SPX_DEV uint32_t chain_len(const SetParams &P, const uint32_t msg[HF::W], int c) {
    auto nib = [&](int i) -> uint32_t {
        // byte i/2 of the value, MSB nibble first
        uint32_t byte;
        if (HF::kShake) byte = (msg[i >> 3] >> (8 * ((i >> 1) & 3))) & 0xffu;
        else byte = (msg[i >> 3] >> (24 - 8 * ((i >> 1) & 3))) & 0xffu;
        return (i & 1) ? (byte & 15u) : (byte >> 4);
    };
    if (c < P.len1) return nib(c);
    uint32_t csum = 0;
    for (int i = 0; i < P.len1; i++) csum += 15u - nib(i);
    const int shift = (8 - ((P.len2 * 4) % 8)) % 8;
    csum <<= shift;
    const int cbits = ((P.len2 * 4 + 7) / 8) * 8;  // checksum bytes as a big-endian integer
    const int j = c - P.len1;
    return (csum >> (cbits - 4 * (j + 1))) & 15u;
}

// Work record of an item from its H_msg digest (hash_sha256.cu:249-261):
// FORS digest, tree and leaf index, and the key's midstate from PUB_SEED.
template <class HF>
SPX_DEV SignWork work_from_digest(const SetParams &P, const uint8_t *dg, const uint8_t *pub) {
    constexpr int N = 4 * HF::W;
    SignWork w;
    for (int j = 0; j < 48; j++) w.mhash[j] = j < P.fors_msg_bytes ? dg[j] : 0;
    uint64_t t = 0;
    for (int j = 0; j < P.tree_bytes; j++) t = (t << 8) | dg[P.fors_msg_bytes + j];
    if (P.tree_bits < 64) t &= (~0ull) >> (64 - P.tree_bits);
    uint32_t l = 0;
    for (int j = 0; j < P.leaf_bytes; j++) l = (l << 8) | dg[P.fors_msg_bytes + P.tree_bytes + j];
    l &= (~0u) >> (32 - P.leaf_bits);
    w.tree = t;
    w.idx_leaf = l;
    w.flags = 0;
    KeyRegs<N> key;
    HF::key_init(key, pub, pub);
#pragma unroll
    for (int j = 0; j < 8; j++) w.mid[j] = key.mid[j];
    return w;
}

// ===========================================================================
// message phase: thread per signature
// ===========================================================================
// Messages of at least long_msg bytes are left to k_sign_msg_pair (0: none).
// The threshold is a kernel argument rather than a field of the argument
// structs: a larger by-value VerifyArgs changed the register allocation of
// the persistent verify kernel and made it ~20% slower.
template <class HF>
__global__ void k_sign_msg(SetParams P, SignArgs A, uint64_t long_msg) {
    constexpr int W = HF::W, N = 4 * W;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.count) return;
    const uint8_t *sk = A.sk.row(i);
    uint32_t skprf[W], opt[W], pk[2 * W], R[W];
    HF::load(skprf, sk + N);
    HF::load(pk, sk + 2 * N);
    HF::load(pk + W, sk + 3 * N);
    if (A.optrand) {
        HF::load(opt, A.optrand + (uint64_t)i * N);
    } else {
#pragma unroll
        for (int j = 0; j < W; j++) opt[j] = 0xadadadadu;
    }
    const uint8_t *m = A.msg.base + A.msg.off[i];
    const uint64_t mlen = A.msg.len[i];
    if (long_msg && mlen >= long_msg) return;   // k_sign_msg_pair / k_sign_msg_wide hash it
    uint8_t dg[64];
    if constexpr (!HF::kShake) {
        HF::msg_digests(R, true, skprf, opt, pk, m, mlen, dg, P.dgst_bytes);
    } else {
        HF::prf_msg(R, skprf, opt, m, mlen);
        HF::h_msg(dg, P.dgst_bytes, R, pk, m, mlen);
    }
    HF::store(A.sig + (uint64_t)i * P.sig_bytes, R);
    A.work[i] = work_from_digest<HF>(P, dg, sk + 2 * N);
}

// Long messages (SHA-256 sets): a 64-thread block takes 32 consecutive items
// and hashes those of at least long_msg bytes with the same PRF_msg and H_msg
// as k_sign_msg, each message pass split between lane l of the schedule warp
// and lane l of the rounds warp (Sha2::stream_msg_pair); shorter items are
// k_sign_msg's.  Per message the issue work is that of one thread, spread
// over two warps, so latency drops without costing throughput.
template <class HF>
__global__ void __launch_bounds__(64) k_sign_msg_pair(SetParams P, SignArgs A, uint64_t long_msg) {
    constexpr int W = HF::W, N = 4 * W;
    __shared__ uint32_t kw[2 * 64 * 32];
    __shared__ uint32_t xr[8 * 32];
    const uint32_t l = threadIdx.x & 31;
    const uint32_t i = blockIdx.x * 32 + l;
    const uint64_t mlen = i < A.count ? A.msg.len[i] : 0;
    const bool mine = i < A.count && mlen >= long_msg;
    // both warps see the same 32 items, so these are uniform over the block
    if (!__any_sync(0xffffffffu, mine)) return;
    const int role = !mine ? 2 : (threadIdx.x < 32 ? 0 : 1);
    uint64_t most = mine ? HF::template msg_blocks<3 * W>(mlen) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t x = __shfl_xor_sync(0xffffffffu, most, o);
        most = x > most ? x : most;
    }
    const uint8_t *sk = mine ? A.sk.row(i) : nullptr;
    const uint8_t *m = mine ? A.msg.base + A.msg.off[i] : nullptr;
    uint32_t skprf[W], opt[W], pre[3 * W], st[8];
#pragma unroll
    for (int j = 0; j < W; j++) skprf[j] = opt[j] = 0xadadadadu;
#pragma unroll
    for (int j = 0; j < 3 * W; j++) pre[j] = 0;
    if (mine) {
        HF::load(skprf, sk + N);
        if (A.optrand) HF::load(opt, A.optrand + (uint64_t)i * N);
    }
    if (role == 1) HF::hmac_start(st, skprf);
    HF::template stream_msg_pair<W>(st, 1, opt, m, mlen, kw, role, most);
    if (role == 1) {
        uint32_t R[W];
        HF::hmac_finish(R, st, skprf);
        HF::store(A.sig + (uint64_t)i * P.sig_bytes, R);
#pragma unroll
        for (int j = 0; j < W; j++) xr[j * 32 + l] = R[j];
    }
    __syncthreads();
    if (mine) {
#pragma unroll
        for (int j = 0; j < W; j++) pre[j] = xr[j * 32 + l];
        HF::load(pre + W, sk + 2 * N);
        HF::load(pre + 2 * W, sk + 3 * N);
    }
    if (role == 1) sha256_iv(st);
    HF::template stream_msg_pair<3 * W>(st, 0, pre, m, mlen, kw, role, most);
    if (role == 1) {
        uint8_t dg[64];
        HF::mgf1_digest(dg, P.dgst_bytes, st);
        A.work[i] = work_from_digest<HF>(P, dg, sk + 2 * N);
    }
}

// Long messages (SHAKE sets): one warp per message.  The sponge of
// PRF_msg = SHAKE256(SK_PRF || optrand || m) and H_msg = SHAKE256(R || PK ||
// m) (hash_shake256.cu:64-77, :96-130) runs with its state spread over the
// warp (warp_keccak_f1600): lane j < 17 loads and absorbs stream lane j of
// each 136-byte block (one coalesced 136-byte read per block, fetched a
// block ahead), and the prefix -- 2n or 3n bytes, whole lanes -- sits in
// lanes below 17 of the first block.  A 1 MiB message is 7,711 serial
// permutations per pass, so a permutation's latency is the message's.
// every lane: stream = prefix (P lanes; lane j < P holds lane j) || m || padding
template <class HF>
SPX_DEV void shake_absorb_warp(uint64_t &a, const KeccakLane &k, uint32_t lane, uint64_t pre, int P,
                               const uint8_t *m, uint64_t mlen) {
    const uint64_t nblocks = (8 * (uint64_t)P + mlen) / 136 + 1;
    auto block_lane = [&](uint64_t b) -> uint64_t {
        const uint64_t q = 17 * b + lane;
        if (lane >= 17) return 0ull;
        if (q < (uint64_t)P) return pre;
        return HF::msg_lane(m, mlen, q - P);   // the 0x1F padding byte included
    };
    a = 0;
    uint64_t nxt = block_lane(0);
    for (uint64_t b = 0; b < nblocks; b++) {
        uint64_t cur = nxt;
        if (b + 1 < nblocks) nxt = block_lane(b + 1);
        if (b + 1 == nblocks && lane == 16) cur ^= 0x8000000000000000ull;
        a ^= cur;
        warp_keccak_f1600(a, k, lane);
    }
}

template <class HF>
__global__ void __launch_bounds__(128) k_sign_msg_wide(SetParams P, SignArgs A, uint64_t long_msg) {
    constexpr int N = 4 * HF::W, NL = N / 8;
    __shared__ uint64_t dgs[4][8];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t i = blockIdx.x * 4 + wib;
    if (i >= A.count) return;                 // warp-uniform
    const uint64_t mlen = A.msg.len[i];
    if (mlen < long_msg) return;              // k_sign_msg hashes it
    KeccakLane k;
    keccak_lane_init(k, lane);
    const uint8_t *sk = A.sk.row(i);
    const uint8_t *m = A.msg.base + A.msg.off[i];
    uint64_t pre = 0, a;
    if (lane < NL) pre = reinterpret_cast<const uint64_t *>(sk + N)[lane];
    else if (lane < 2 * NL)
        pre = A.optrand ? reinterpret_cast<const uint64_t *>(A.optrand + (uint64_t)i * N)[lane - NL]
                        : 0xadadadadadadadadull;   // the reference's fixed optrand (sign.cu:1950-1954)
    shake_absorb_warp<HF>(a, k, lane, pre, 2 * NL, m, mlen);
    if (lane < NL) reinterpret_cast<uint64_t *>(A.sig + (uint64_t)i * P.sig_bytes)[lane] = a;   // R
    pre = lane < NL ? a : (lane < 3 * NL ? reinterpret_cast<const uint64_t *>(sk + 2 * N)[lane - NL] : 0ull);
    shake_absorb_warp<HF>(a, k, lane, pre, 3 * NL, m, mlen);
    if (lane < 8) dgs[wib][lane] = a;
    __syncwarp();
    if (lane == 0) A.work[i] = work_from_digest<HF>(P, reinterpret_cast<const uint8_t *>(dgs[wib]), sk + 2 * N);
}

// ===========================================================================
// FORS sign: a group of G = 2^g lanes per (signature, tree), g in 0..5.  Lane
// l of a group owns the contiguous subtree of 2^(a-g) leaves starting at
// l*2^(a-g) and reduces it with a shared-memory stack (treehash,
// utils.cu:189-241); the G subtree roots are then reduced over g shuffle
// levels inside the group.  g = 0 is one lane per tree (no idle lanes in the
// reduction, best for big batches); g = 5 is one warp per tree (lowest
// latency, best for few signatures or tall trees).  Auth-path nodes are
// written by whichever lane holds them.
// ===========================================================================
template <class HF>
__global__ void k_fors_sign(SetParams P, SignArgs A, int g) {
    constexpr int W = HF::W, N = 4 * W;
    extern __shared__ uint32_t smem[];
    const uint32_t G = 1u << g;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = (uint32_t)(gid & (G - 1));
    uint64_t tid = gid >> g;
    const uint64_t ntrees = (uint64_t)A.count * P.k;
    // every lane of a warp takes part in the shuffles; lanes past the end work
    // on tree 0 and store nothing
    const bool valid = tid < ntrees;
    if (!valid) tid = 0;
    const uint32_t item = (uint32_t)(tid / P.k);
    const int t = (int)(tid % P.k);
    const SignWork wk = A.work[item];
    const uint8_t *sk = A.sk.row(item);
    KeyRegs<N> key;
    key_from_work<HF>(key, sk, sk + 2 * N, wk);
    const uint32_t idx = fors_index(wk.mhash, P.a, t);
    const int sub = P.a - g;                    // lane subtree height
    const uint32_t per = 1u << sub;
    const uint32_t off = (uint32_t)t << P.a;   // idx_offset
    uint8_t *sigt = A.sig + (uint64_t)item * P.sig_bytes + N + (uint64_t)t * (P.a + 1) * N;

    Adrs ad;  // FORS tree address: layer 0, tree, key pair idx_leaf, type FORSTREE
    adrs_zero(ad);
    adrs_tree(ad, wk.tree);
    adrs_keypair(ad, wk.idx_leaf);
    adrs_type(ad, ADDR_FORSTREE);

    // per-lane stack: sub+1 entries of W words (heights in registers/local)
    uint32_t *stk = smem + threadIdx.x * (sub + 1) * W;
    int heights[17];
    int sp = 0;
    uint32_t v[W];
    for (uint32_t jj = 0; jj < per; jj++) {
        const uint32_t j = lane * per + jj;
        adrs_height(ad, 0);
        adrs_index(ad, off + j);
        uint32_t skv[W];
        HF::PRF(skv, ad, key);
        if (valid && j == idx) HF::store(sigt, skv);
        HF::F(v, skv, ad, key);
        if (valid && (idx ^ 1u) == j) HF::store(sigt + N, v);
        int hgt = 0;
        // merge equal-height nodes on the stack
        while (sp > 0 && heights[sp - 1] == hgt) {
            uint32_t l[W];
#pragma unroll
            for (int q = 0; q < W; q++) l[q] = stk[(sp - 1) * W + q];
            const uint32_t tidx = j >> (hgt + 1);
            adrs_height(ad, hgt + 1);
            adrs_index(ad, tidx + (off >> (hgt + 1)));
            HF::H(v, l, v, ad, key);
            sp--;
            hgt++;
            if (valid && ((idx >> hgt) ^ 1u) == tidx) HF::store(sigt + N + (uint64_t)hgt * N, v);
        }
#pragma unroll
        for (int q = 0; q < W; q++) stk[sp * W + q] = v[q];
        heights[sp] = hgt;
        sp++;
    }
    // v = this lane's subtree root at height `sub`, index lane
    for (int s = 0; s < g; s++) {
        const int hgt = sub + s;
        const uint32_t q = lane >> s;
        const bool holder = (lane & ((1u << s) - 1)) == 0;
        if (valid && holder && ((idx >> hgt) ^ 1u) == q) HF::store(sigt + N + (uint64_t)hgt * N, v);
        uint32_t r[W];
#pragma unroll
        for (int x = 0; x < W; x++) r[x] = __shfl_down_sync(0xffffffffu, v[x], 1u << s, G);
        if ((lane & ((2u << s) - 1)) == 0) {
            adrs_height(ad, hgt + 1);
            adrs_index(ad, (q >> 1) + (off >> (hgt + 1)));
            HF::H(v, v, r, ad, key);
        }
    }
    if (valid && lane == 0) HF::store(A.fors_roots + ((uint64_t)item * P.k + t) * N, v);
}

// ===========================================================================
// XMSS leaves: one thread per (item, layer, leaf).  WOTS+ public key
// (wots_gen_pk, wots.cu:176-185) streamed straight into T_len (the leaf,
// sign.cu:87-102).  The signing leaf of each layer also records every chain
// value so the WOTS signature (wots_sign, wots.cu:614-625) is a gather.
// ===========================================================================
struct LeafArgs {
    uint32_t count;      // items
    int layer0;          // first layer handled
    int nlayers;         // layers per item
    KeyRef sk;
    const SignWork *work;  // null for key generation (tree 0, no signing leaf)
    uint8_t *leaves;     // [item][layer-layer0][leaf] n bytes
    uint8_t *chains;     // [item][layer][chain][16] n bytes, or null
    uint8_t *ends;       // chain-parallel mode: [item][layer-layer0][leaf][chain] n bytes
};

template <class HF>
__global__ void __launch_bounds__(256, HF::kLeafMinBlocks) k_leaves(SetParams P, LeafArgs A) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    extern __shared__ uint32_t smem[];
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nleaf = 1u << P.hp;
    if (gid >= (uint64_t)A.count * A.nlayers * nleaf) return;
    const uint32_t item = (uint32_t)(gid / ((uint64_t)A.nlayers * nleaf));
    const uint32_t rem = (uint32_t)(gid % ((uint64_t)A.nlayers * nleaf));
    const int L = A.layer0 + (int)(rem >> P.hp);
    const uint32_t j = rem & (nleaf - 1);
    const uint8_t *sk = A.sk.row(item);
    KeyRegs<N> key;
    uint64_t tree_L = 0;
    uint32_t idx_L = 0xffffffffu;
    if (A.work) {
        const SignWork wk = A.work[item];
        key_from_work<HF>(key, sk, sk + 2 * N, wk);
        layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    } else {
        HF::key_init(key, sk, sk + 2 * N);
    }
    const bool rec = A.chains && (j == idx_L);
    uint8_t *chain = rec ? A.chains + (((uint64_t)item * P.d + L) * LEN) * 16 * N : nullptr;

    Adrs wa, pa;
    adrs_zero(wa);
    adrs_layer(wa, L);
    adrs_tree(wa, tree_L);
    adrs_type(wa, ADDR_WOTS);
    adrs_keypair(wa, j);
    adrs_zero(pa);
    adrs_copy_keypair(pa, wa);
    adrs_type(pa, ADDR_WOTSPK);

    typename HF::TStream ts;
    HF::t_init(ts, smem + threadIdx.x * HF::kSmemWords, key, pa);
    for (int c = 0; c < LEN; c++) {
        uint32_t v[W];
        adrs_chain(wa, c);
        adrs_hash(wa, 0);
        HF::PRF(v, wa, key);
        if (rec) HF::store(chain + ((uint64_t)c * 16) * N, v);
        typename HF::FCtx fc;
        HF::f_prepare(fc, wa, key);
        for (int s = 0; s < 15; s++) {
            HF::f_step(v, v, fc, s, key);
            if (rec) HF::store(chain + ((uint64_t)c * 16 + s + 1) * N, v);
        }
        HF::t_absorb(ts, v, key);
    }
    uint32_t leaf[W];
    HF::t_final(leaf, ts);
    HF::store(A.leaves + (((uint64_t)item * A.nlayers + (L - A.layer0)) * nleaf + j) * N, leaf);
}

// ===========================================================================
// XMSS leaves, chain-parallel mode (small batches): one thread per WOTS+
// chain (wots_gen_pk's loop body, wots.cu:181-184) writes its chain end;
// then one thread per leaf hashes the len ends with T_len.  35x (n=16) the
// threads of k_leaves, so a few signatures still fill the GPU; the cost is
// the chain-end round trip through memory and an idle T_len pass for most
// lanes, which is why big batches use k_leaves.
// ===========================================================================
template <class HF>
__global__ void k_leaf_chains(SetParams P, LeafArgs A) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nleaf = 1u << P.hp;
    const uint64_t per_item = (uint64_t)A.nlayers * nleaf * LEN;
    if (gid >= (uint64_t)A.count * per_item) return;
    const uint32_t item = (uint32_t)(gid / per_item);
    uint32_t rem = (uint32_t)(gid % per_item);
    const int c = (int)(rem % LEN);
    rem /= LEN;
    const uint32_t j = rem & (nleaf - 1);
    const int Lr = (int)(rem >> P.hp);
    const int L = A.layer0 + Lr;
    const uint8_t *sk = A.sk.row(item);
    KeyRegs<N> key;
    uint64_t tree_L = 0;
    uint32_t idx_L = 0xffffffffu;
    if (A.work) {
        const SignWork wk = A.work[item];
        key_from_work<HF>(key, sk, sk + 2 * N, wk);
        layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    } else {
        HF::key_init(key, sk, sk + 2 * N);
    }
    const bool rec = A.chains && (j == idx_L);
    uint8_t *chain = rec ? A.chains + ((((uint64_t)item * P.d + L) * LEN + c) * 16) * N : nullptr;
    Adrs wa;
    adrs_zero(wa);
    adrs_layer(wa, L);
    adrs_tree(wa, tree_L);
    adrs_type(wa, ADDR_WOTS);
    adrs_keypair(wa, j);
    adrs_chain(wa, c);
    adrs_hash(wa, 0);
    uint32_t v[W];
    HF::PRF(v, wa, key);
    if (rec) HF::store(chain, v);
    typename HF::FCtx fc;
    HF::f_prepare(fc, wa, key);
    for (int s = 0; s < 15; s++) {
        HF::f_step(v, v, fc, s, key);
        if (rec) HF::store(chain + (uint64_t)(s + 1) * N, v);
    }
    HF::store(A.ends + gid * N, v);
}

// T_l of m n-byte values in global memory under ADRS pa into out, by one
// thread over a slot of `VsortSmem<HF>::slot_stride(0)` shared words
// (spx_vsort.cuh): the values staged with their loads in flight together,
// then the hash unit by unit through one call site.
template <class HF>
SPX_DEV void slot_tl(uint32_t *S, const KeyRegs<4 * HF::W> &key, const uint8_t *pub, const Adrs &pa,
                     const uint8_t *vals, int m, uint32_t out[HF::W]);

// thread per WOTS+ leaf: T_len over its chain ends, through a slot of
// slot_words shared words per thread (slot_tl; small sign batches, where the
// thread's serial latency is what counts), or with slot_words 0 through the
// T stream of HF::kSmemWords shared words per thread (key generation's
// large batches, where the smaller footprint keeps more warps resident).
template <class HF>
__global__ void k_leaf_tlen(SetParams P, LeafArgs A, uint32_t slot_words) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    extern __shared__ uint32_t smem[];
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nleaf = 1u << P.hp;
    if (gid >= (uint64_t)A.count * A.nlayers * nleaf) return;
    const uint32_t item = (uint32_t)(gid / ((uint64_t)A.nlayers * nleaf));
    const uint32_t rem = (uint32_t)(gid % ((uint64_t)A.nlayers * nleaf));
    const int L = A.layer0 + (int)(rem >> P.hp);
    const uint32_t j = rem & (nleaf - 1);
    const uint8_t *sk = A.sk.row(item);
    KeyRegs<N> key;
    uint64_t tree_L = 0;
    uint32_t idx_L = 0;
    if (A.work) {
        const SignWork wk = A.work[item];
        key_from_work<HF>(key, sk, sk + 2 * N, wk);
        layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    } else {
        HF::key_init(key, sk, sk + 2 * N);
    }
    Adrs pa;
    adrs_zero(pa);
    adrs_layer(pa, L);
    adrs_tree(pa, tree_L);
    adrs_type(pa, ADDR_WOTSPK);
    adrs_keypair(pa, j);
    uint32_t leaf[W];
    const uint8_t *e = A.ends + gid * LEN * N;
    if (slot_words) {
        slot_tl<HF>(smem + threadIdx.x * slot_words, key, sk + 2 * N, pa, e, LEN, leaf);
    } else {
        typename HF::TStream ts;
        HF::t_init(ts, smem + threadIdx.x * HF::kSmemWords, key, pa);
        for (int c = 0; c < LEN; c++) {
            uint32_t v[W];
            HF::load(v, e + (uint64_t)c * N);
            HF::t_absorb(ts, v, key);
        }
        HF::t_final(leaf, ts);
    }
    HF::store(A.leaves + gid * N, leaf);
}

// ===========================================================================
// XMSS trees: one warp per (item, layer); the 2^hp leaves are reduced level
// by level in shared memory (treehash node addresses, utils.cu:209-233).
// Writes the auth path of the layer's signing leaf (or none for keygen) and
// the root.
// ===========================================================================
struct TreeArgs {
    uint32_t count;
    int layer0, nlayers;
    KeyRef sk;
    const SignWork *work;   // null for key generation
    const uint8_t *leaves;
    uint8_t *roots;         // [item][layer-layer0] n bytes
    uint8_t *sig;           // auth paths are written here when work != null
};

// Lane-per-tree variant for short subtrees: a thread reduces one whole
// (item, layer) tree with a stack of hp+1 nodes; no shared memory, no idle
// lanes in the upper levels.
template <class HF>
__global__ void k_trees_lane(SetParams P, TreeArgs A) {
    constexpr int W = HF::W, N = 4 * W;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)A.count * A.nlayers) return;
    const uint32_t item = (uint32_t)(gid / A.nlayers);
    const int L = A.layer0 + (int)(gid % A.nlayers);
    const uint32_t nleaf = 1u << P.hp;
    const uint8_t *sk = A.sk.row(item);
    KeyRegs<N> key;
    uint64_t tree_L = 0;
    uint32_t idx_L = 0;
    if (A.work) {
        const SignWork wk = A.work[item];
        key_from_work<HF>(key, sk, sk + 2 * N, wk);
        layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    } else {
        HF::key_init(key, sk, sk + 2 * N);
    }
    const uint8_t *lv = A.leaves + (((uint64_t)item * A.nlayers + (L - A.layer0)) * nleaf) * N;
    uint8_t *auth = nullptr;
    if (A.work)
        auth = A.sig + (uint64_t)item * P.sig_bytes + N + P.fors_bytes +
               (uint64_t)L * (P.wots_bytes + P.hp * N) + P.wots_bytes;
    Adrs ad;
    adrs_zero(ad);
    adrs_layer(ad, L);
    adrs_tree(ad, tree_L);
    adrs_type(ad, ADDR_HASHTREE);
    uint32_t stk[5][W];   // hp <= 4 in this variant
    int heights[5];
    int sp = 0;
    for (uint32_t j = 0; j < nleaf; j++) {
        uint32_t v[W];
        HF::load(v, lv + (uint64_t)j * N);
        if (auth && (idx_L ^ 1u) == j) HF::store(auth, v);
        int hgt = 0;
        while (sp > 0 && heights[sp - 1] == hgt) {
            const uint32_t tidx = j >> (hgt + 1);
            adrs_height(ad, hgt + 1);
            adrs_index(ad, tidx);
            uint32_t l[W];
#pragma unroll
            for (int x = 0; x < W; x++) l[x] = stk[sp - 1][x];
            HF::H(v, l, v, ad, key);
            sp--;
            hgt++;
            if (auth && hgt < P.hp && ((idx_L >> hgt) ^ 1u) == tidx) HF::store(auth + (uint64_t)hgt * N, v);
        }
#pragma unroll
        for (int x = 0; x < W; x++) stk[sp][x] = v[x];
        heights[sp] = hgt;
        sp++;
    }
    uint32_t root[W];
#pragma unroll
    for (int x = 0; x < W; x++) root[x] = stk[0][x];
    HF::store(A.roots + ((uint64_t)item * A.nlayers + (L - A.layer0)) * N, root);
}

template <class HF>
__global__ void k_trees(SetParams P, TreeArgs A) {
    constexpr int W = HF::W, N = 4 * W;
    extern __shared__ uint32_t smem[];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= (uint64_t)A.count * A.nlayers) return;
    const uint32_t item = (uint32_t)(gw / A.nlayers);
    const int L = A.layer0 + (int)(gw % A.nlayers);
    const uint32_t nleaf = 1u << P.hp;
    uint32_t *nodes = smem + wib * (2 * nleaf * W);   // level l at offset (2*nleaf - 2*(nleaf>>l))
    const uint8_t *sk = A.sk.row(item);
    KeyRegs<N> key;
    uint64_t tree_L = 0;
    uint32_t idx_L = 0;
    if (A.work) {
        const SignWork wk = A.work[item];
        key_from_work<HF>(key, sk, sk + 2 * N, wk);
        layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    } else {
        HF::key_init(key, sk, sk + 2 * N);
    }
    const uint8_t *lv = A.leaves + (((uint64_t)item * A.nlayers + (L - A.layer0)) * nleaf) * N;
    for (uint32_t q = lane; q < nleaf; q += 32) {
        uint32_t v[W];
        HF::load(v, lv + (uint64_t)q * N);
#pragma unroll
        for (int x = 0; x < W; x++) nodes[q * W + x] = v[x];
    }
    __syncwarp();
    uint8_t *auth = nullptr;
    if (A.work)
        auth = A.sig + (uint64_t)item * P.sig_bytes + N + P.fors_bytes +
               (uint64_t)L * (P.wots_bytes + P.hp * N) + P.wots_bytes;
    Adrs ad;
    adrs_zero(ad);
    adrs_layer(ad, L);
    adrs_tree(ad, tree_L);
    adrs_type(ad, ADDR_HASHTREE);
    uint32_t base = 0;  // offset (in nodes) of the current level
    for (int h = 0; h < P.hp; h++) {
        const uint32_t cnt = nleaf >> h;
        if (auth && lane == 0) {
            uint32_t v[W];
            const uint32_t sib = (idx_L >> h) ^ 1u;
#pragma unroll
            for (int x = 0; x < W; x++) v[x] = nodes[(base + sib) * W + x];
            HF::store(auth + (uint64_t)h * N, v);
        }
        const uint32_t nb = base + cnt;
        for (uint32_t q = lane; q < cnt / 2; q += 32) {
            uint32_t l[W], r[W], o[W];
#pragma unroll
            for (int x = 0; x < W; x++) {
                l[x] = nodes[(base + 2 * q) * W + x];
                r[x] = nodes[(base + 2 * q + 1) * W + x];
            }
            adrs_height(ad, h + 1);
            adrs_index(ad, q);
            HF::H(o, l, r, ad, key);
#pragma unroll
            for (int x = 0; x < W; x++) nodes[(nb + q) * W + x] = o[x];
        }
        __syncwarp();
        base = nb;
    }
    if (lane == 0) {
        uint32_t v[W];
#pragma unroll
        for (int x = 0; x < W; x++) v[x] = nodes[base * W + x];
        HF::store(A.roots + ((uint64_t)item * A.nlayers + (L - A.layer0)) * N, v);
    }
}

// ===========================================================================
// sign finish: block per signature.  Thread 0 computes the FORS public key
// T_k(roots) (fors.cu:141-142); then all threads gather each layer's WOTS
// signature from the recorded chain values: layer 0 signs the FORS key,
// layer L signs the root of layer L-1.
// ===========================================================================
template <class HF>
__global__ void k_sign_finish(SetParams P, SignArgs A) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    extern __shared__ uint32_t smem[];
    const uint32_t item = blockIdx.x;
    if (item >= A.count) return;
    uint32_t *forspk = smem;                   // W words
    uint32_t *slot = smem + 8;                 // slot_tl scratch
    const SignWork wk = A.work[item];
    const uint8_t *sk = A.sk.row(item);
    if (threadIdx.x == 0) {
        KeyRegs<N> key;
        key_from_work<HF>(key, sk, sk + 2 * N, wk);
        Adrs pa;
        adrs_zero(pa);
        adrs_tree(pa, wk.tree);
        adrs_keypair(pa, wk.idx_leaf);
        adrs_type(pa, ADDR_FORSPK);
        uint32_t o[W];
        slot_tl<HF>(slot, key, sk + 2 * N, pa, A.fors_roots + (uint64_t)item * P.k * N, P.k, o);
#pragma unroll
        for (int x = 0; x < W; x++) forspk[x] = o[x];
        // the top layer root must equal the key's root; otherwise the key row
        // is inconsistent (sk root does not match its seeds)
        uint32_t top[W], skroot[W];
        HF::load(top, A.roots + ((uint64_t)item * P.d + (P.d - 1)) * N);
        HF::load(skroot, sk + 3 * N);
        bool ok = true;
#pragma unroll
        for (int x = 0; x < W; x++) ok &= top[x] == skroot[x];
        if (A.status) A.status[item] = ok ? 0 : -2;
    }
    __syncthreads();
    uint8_t *sig = A.sig + (uint64_t)item * P.sig_bytes;
    for (int e = threadIdx.x; e < P.d * LEN; e += blockDim.x) {
        const int L = e / LEN, c = e % LEN;
        uint32_t msg[W];
        if (L == 0) {
#pragma unroll
            for (int x = 0; x < W; x++) msg[x] = forspk[x];
        } else {
            HF::load(msg, A.roots + ((uint64_t)item * P.d + (L - 1)) * N);
        }
        const uint32_t ln = chain_len<HF>(P, msg, c);
        const uint8_t *src = A.chains + ((((uint64_t)item * P.d + L) * LEN + c) * 16 + ln) * N;
        uint32_t v[W];
        load_bytes_le<N>(v, src);
        store_bytes_le<N>(sig + N + P.fors_bytes + (uint64_t)L * (P.wots_bytes + P.hp * N) + (uint64_t)c * N, v);
    }
}

// ===========================================================================
// verify
// ===========================================================================
struct VerifyArgs {
    uint32_t count;
    KeyRef pk;
    MsgRef msg;
    const uint8_t *sig;         // count x sig_bytes (row stride sig_stride)
    uint64_t sig_stride;
    const uint64_t *siglen;     // per item, or null = sig_bytes
    SignWork *work;
    uint8_t *fors_roots;        // count x k x n
    int32_t *verdict;           // 0 accept, -1 reject (crypto_sign_verify)
    uint8_t *wpk;               // count x len x n: WOTS public key of the current layer
    uint8_t *cur_root;          // count x n: root of the layer below (FORS key for layer 0)
    uint32_t *ctr = nullptr;    // persistent verify: next item to take (zeroed per launch)
};

template <class HF>
__global__ void k_verify_msg(SetParams P, VerifyArgs A, uint64_t long_msg) {
    constexpr int W = HF::W, N = 4 * W;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.count) return;
    SignWork w;
    w.flags = 0;
    if (A.siglen && A.siglen[i] != (uint64_t)P.sig_bytes) {
        w.flags = 1;  // wrong length: reject without hashing (sign.cu:3063-3065)
        w.tree = 0;
        w.idx_leaf = 0;
        for (int j = 0; j < 48; j++) w.mhash[j] = 0;
        A.work[i] = w;
        return;
    }
    if (long_msg && A.msg.len[i] >= long_msg) return;   // k_verify_msg_pair / _wide hash it
    const uint8_t *pkb = A.pk.row(i);
    const uint8_t *sig = A.sig + (uint64_t)i * A.sig_stride;
    uint32_t R[W], pk[2 * W];
    HF::load(R, sig);
    HF::load(pk, pkb);
    HF::load(pk + W, pkb + N);
    uint8_t dg[64];
    if constexpr (!HF::kShake) HF::msg_digests(R, false, R, R, pk, A.msg.base + A.msg.off[i], A.msg.len[i], dg,
                                               P.dgst_bytes);
    else HF::h_msg(dg, P.dgst_bytes, R, pk, A.msg.base + A.msg.off[i], A.msg.len[i]);
    A.work[i] = work_from_digest<HF>(P, dg, pkb);
}

// H_msg of long messages over two warps (SHA-256 sets), 32 items per
// block as in k_sign_msg_pair
template <class HF>
__global__ void __launch_bounds__(64) k_verify_msg_pair(SetParams P, VerifyArgs A, uint64_t long_msg) {
    constexpr int W = HF::W, N = 4 * W;
    __shared__ uint32_t kw[2 * 64 * 32];
    const uint32_t l = threadIdx.x & 31;
    const uint32_t i = blockIdx.x * 32 + l;
    const uint64_t mlen = i < A.count ? A.msg.len[i] : 0;
    // wrong-length signatures were rejected by k_verify_msg without hashing
    const bool mine = i < A.count && mlen >= long_msg && !(A.siglen && A.siglen[i] != (uint64_t)P.sig_bytes);
    if (!__any_sync(0xffffffffu, mine)) return;   // uniform over the block
    const int role = !mine ? 2 : (threadIdx.x < 32 ? 0 : 1);
    uint64_t most = mine ? HF::template msg_blocks<3 * W>(mlen) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t x = __shfl_xor_sync(0xffffffffu, most, o);
        most = x > most ? x : most;
    }
    const uint8_t *pkb = mine ? A.pk.row(i) : nullptr;
    uint32_t pre[3 * W], st[8];
#pragma unroll
    for (int j = 0; j < 3 * W; j++) pre[j] = 0;
    if (mine) {
        HF::load(pre, A.sig + (uint64_t)i * A.sig_stride);
        HF::load(pre + W, pkb);
        HF::load(pre + 2 * W, pkb + N);
    }
    if (role == 1) sha256_iv(st);
    HF::template stream_msg_pair<3 * W>(st, 0, pre, mine ? A.msg.base + A.msg.off[i] : nullptr, mlen, kw, role,
                                        most);
    if (role == 1) {
        uint8_t dg[64];
        HF::mgf1_digest(dg, P.dgst_bytes, st);
        A.work[i] = work_from_digest<HF>(P, dg, pkb);
    }
}

// H_msg of long messages (SHAKE sets): one warp per message, as in
// k_sign_msg_wide
template <class HF>
__global__ void __launch_bounds__(128) k_verify_msg_wide(SetParams P, VerifyArgs A, uint64_t long_msg) {
    constexpr int N = 4 * HF::W, NL = N / 8;
    __shared__ uint64_t dgs[4][8];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t i = blockIdx.x * 4 + wib;
    if (i >= A.count) return;                                           // warp-uniform
    if (A.siglen && A.siglen[i] != (uint64_t)P.sig_bytes) return;      // rejected by k_verify_msg
    const uint64_t mlen = A.msg.len[i];
    if (mlen < long_msg) return;                                        // k_verify_msg hashes it
    KeccakLane k;
    keccak_lane_init(k, lane);
    const uint8_t *pkb = A.pk.row(i);
    const uint8_t *sig = A.sig + (uint64_t)i * A.sig_stride;
    uint64_t a;
    const uint64_t pre = lane < NL ? reinterpret_cast<const uint64_t *>(sig)[lane]
                                   : (lane < 3 * NL ? reinterpret_cast<const uint64_t *>(pkb)[lane - NL] : 0ull);
    shake_absorb_warp<HF>(a, k, lane, pre, 3 * NL, A.msg.base + A.msg.off[i], mlen);
    if (lane < 8) dgs[wib][lane] = a;
    __syncwarp();
    if (lane == 0) A.work[i] = work_from_digest<HF>(P, reinterpret_cast<const uint8_t *>(dgs[wib]), pkb);
}

// root from a leaf and its auth path (compute_root, utils.cu:94-135)
template <class HF>
SPX_DEV void compute_root(uint32_t root[HF::W], const uint32_t leaf[HF::W], uint32_t leaf_idx, uint32_t idx_offset,
                          const uint8_t *auth, int height, Adrs &ad, const KeyRegs<4 * HF::W> &key) {
    constexpr int W = HF::W, N = 4 * W;
    uint32_t cur[W];
#pragma unroll
    for (int x = 0; x < W; x++) cur[x] = leaf[x];
    for (int i = 0; i < height; i++) {
        uint32_t sib[W];
        HF::load(sib, auth + (uint64_t)i * N);
        const bool right = leaf_idx & 1u;
        leaf_idx >>= 1;
        idx_offset >>= 1;
        adrs_height(ad, i + 1);
        adrs_index(ad, leaf_idx + idx_offset);
        if (right) HF::H(cur, sib, cur, ad, key);
        else HF::H(cur, cur, sib, ad, key);
    }
#pragma unroll
    for (int x = 0; x < W; x++) root[x] = cur[x];
}

// FORS roots from the signature: thread per (item, tree) of items
// [first, first + n) (fors_pk_from_sig, fors.cu:596-631)
template <class HF>
__global__ void k_verify_fors(SetParams P, VerifyArgs A, uint32_t first, uint32_t n) {
    constexpr int W = HF::W, N = 4 * W;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)n * P.k) return;
    const uint32_t item = first + (uint32_t)(gid / P.k);
    const int t = (int)(gid % P.k);
    const SignWork wk = A.work[item];
    if (wk.flags) return;
    const uint8_t *pkb = A.pk.row(item);
    KeyRegs<N> key;
    key_from_work<HF>(key, pkb, pkb, wk);   // verify needs PUB_SEED only
    const uint32_t idx = fors_index(wk.mhash, P.a, t);
    const uint32_t off = (uint32_t)t << P.a;
    const uint8_t *st = A.sig + (uint64_t)item * A.sig_stride + N + (uint64_t)t * (P.a + 1) * N;
    Adrs ad;
    adrs_zero(ad);
    adrs_tree(ad, wk.tree);
    adrs_keypair(ad, wk.idx_leaf);
    adrs_type(ad, ADDR_FORSTREE);
    adrs_height(ad, 0);
    adrs_index(ad, idx + off);
    uint32_t skv[W], leaf[W], root[W];
    HF::load(skv, st);
    HF::F(leaf, skv, ad, key);
    compute_root<HF>(root, leaf, idx, off, st + N, P.a, ad, key);
    HF::store(A.fors_roots + ((uint64_t)item * P.k + t) * N, root);
}

// hypertree: thread per item, serial over the d layers (the verifier's
// data dependency: layer L signs the root of layer L-1)
template <class HF>
__global__ void k_verify_ht(SetParams P, VerifyArgs A) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    extern __shared__ uint32_t smem[];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.count) return;
    const SignWork wk = A.work[i];
    if (wk.flags) {
        A.verdict[i] = -1;
        return;
    }
    const uint8_t *pkb = A.pk.row(i);
    KeyRegs<N> key;
    key_from_work<HF>(key, pkb, pkb, wk);
    uint32_t *tb = smem + threadIdx.x * HF::kSmemWords;
    uint32_t root[W];
    {
        Adrs pa;
        adrs_zero(pa);
        adrs_tree(pa, wk.tree);
        adrs_keypair(pa, wk.idx_leaf);
        adrs_type(pa, ADDR_FORSPK);
        typename HF::TStream ts;
        HF::t_init(ts, tb, key, pa);
        for (int t = 0; t < P.k; t++) {
            uint32_t v[W];
            HF::load(v, A.fors_roots + ((uint64_t)i * P.k + t) * N);
            HF::t_absorb(ts, v, key);
        }
        HF::t_final(root, ts);
    }
    const uint8_t *sig = A.sig + (uint64_t)i * A.sig_stride + N + P.fors_bytes;
    for (int L = 0; L < P.d; L++) {
        uint64_t tree_L;
        uint32_t idx_L;
        layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
        Adrs wa, pa;
        adrs_zero(wa);
        adrs_layer(wa, L);
        adrs_tree(wa, tree_L);
        adrs_type(wa, ADDR_WOTS);
        adrs_keypair(wa, idx_L);
        adrs_zero(pa);
        adrs_copy_keypair(pa, wa);
        adrs_type(pa, ADDR_WOTSPK);
        typename HF::TStream ts;
        HF::t_init(ts, tb, key, pa);
        for (int c = 0; c < LEN; c++) {
            uint32_t v[W];
            HF::load(v, sig + (uint64_t)c * N);
            const uint32_t ln = chain_len<HF>(P, root, c);
            adrs_chain(wa, c);
            typename HF::FCtx fc;
            HF::f_prepare(fc, wa, key);
            for (uint32_t s = ln; s < 15; s++) HF::f_step(v, v, fc, s, key);
            HF::t_absorb(ts, v, key);
        }
        uint32_t leaf[W];
        HF::t_final(leaf, ts);
        Adrs ta;
        adrs_zero(ta);
        adrs_layer(ta, L);
        adrs_tree(ta, tree_L);
        adrs_type(ta, ADDR_HASHTREE);
        compute_root<HF>(root, leaf, idx_L, 0, sig + P.wots_bytes, P.hp, ta, key);
        sig += P.wots_bytes + P.hp * N;
    }
    uint32_t pr[W];
    HF::load(pr, pkb + N);
    bool ok = true;
#pragma unroll
    for (int x = 0; x < W; x++) ok &= pr[x] == root[x];
    A.verdict[i] = ok ? 0 : -1;
}

// ---------------------------------------------------------------------------
// Layered verify.  The verifier is serial over the d layers (layer L signs
// the root of layer L-1), so each layer is two flat kernels over the whole
// batch instead of one thread walking all layers:
//   k_verify_chains  every (item, chain) pair: finish the WOTS+ chain from the
//                    signature value (wots_pk_from_sig, wots.cu:777-789)
//   k_verify_root    thread per item: T_len over the chain ends, then the
//                    subtree root from the auth path (sign.cu:3103-3109);
//                    with L = -1 it computes the FORS key T_k instead, and at
//                    L = d-1 it compares with PK.root (sign.cu:3116)
// ---------------------------------------------------------------------------
// Root of layer L of an item into root[]: L = -1 the FORS key T_k over the
// k FORS roots at `vals`; otherwise T_len over the len WOTS+ public-key
// values at `vals`, then the subtree root from the auth path at `auth`.  The
// values and the auth path may sit in global or shared memory.  tb: the
// thread's T stream scratch of HF::kSmemWords shared words.
template <class HF>
SPX_DEV void verify_layer_root(const SetParams &P, const SignWork &wk, const KeyRegs<4 * HF::W> &key, int L,
                               uint32_t *tb, const uint8_t *vals, const uint8_t *auth, uint32_t root[HF::W]) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    typename HF::TStream ts;
    if (L < 0) {
        Adrs pa;
        adrs_zero(pa);
        adrs_tree(pa, wk.tree);
        adrs_keypair(pa, wk.idx_leaf);
        adrs_type(pa, ADDR_FORSPK);
        HF::t_init(ts, tb, key, pa);
        for (int t = 0; t < P.k; t++) {
            uint32_t v[W];
            HF::load(v, vals + (uint64_t)t * N);
            HF::t_absorb(ts, v, key);
        }
        HF::t_final(root, ts);
        return;
    }
    uint64_t tree_L;
    uint32_t idx_L;
    layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
    Adrs pa;
    adrs_zero(pa);
    adrs_layer(pa, L);
    adrs_tree(pa, tree_L);
    adrs_keypair(pa, idx_L);
    adrs_type(pa, ADDR_WOTSPK);
    HF::t_init(ts, tb, key, pa);
    for (int c = 0; c < LEN; c++) {
        uint32_t v[W];
        HF::load(v, vals + (uint64_t)c * N);
        HF::t_absorb(ts, v, key);
    }
    uint32_t leaf[W];
    HF::t_final(leaf, ts);
    Adrs ta;
    adrs_zero(ta);
    adrs_layer(ta, L);
    adrs_tree(ta, tree_L);
    adrs_type(ta, ADDR_HASHTREE);
    compute_root<HF>(root, leaf, idx_L, 0, auth, P.hp, ta, key);
}

// offset of layer L's WOTS+ signature in a signature (sign.cu:3092-3110);
// its auth path follows at + wots_bytes
SPX_DEV uint64_t sig_layer_off(const SetParams &P, int L) {
    return (uint64_t)P.n + P.fors_bytes + (uint64_t)L * (P.wots_bytes + (uint64_t)P.hp * P.n);
}

template <class HF>
__global__ void k_verify_root(SetParams P, VerifyArgs A, int L) {
    constexpr int W = HF::W, N = 4 * W;
    extern __shared__ uint32_t smem[];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.count) return;
    const SignWork wk = A.work[i];
    if (wk.flags) {
        if (L == P.d - 1) A.verdict[i] = -1;
        return;
    }
    const uint8_t *pkb = A.pk.row(i);
    KeyRegs<N> key;
    key_from_work<HF>(key, pkb, pkb, wk);
    constexpr int LEN = 2 * N + 3;
    const uint8_t *vals = L < 0 ? A.fors_roots + (uint64_t)i * P.k * N : A.wpk + (uint64_t)i * LEN * N;
    const uint8_t *auth = A.sig + (uint64_t)i * A.sig_stride + (L < 0 ? 0 : sig_layer_off(P, L) + P.wots_bytes);
    uint32_t root[W];
    verify_layer_root<HF>(P, wk, key, L, smem + threadIdx.x * HF::kSmemWords, vals, auth, root);
    if (L == P.d - 1) {
        uint32_t pr[W];
        HF::load(pr, pkb + N);
        bool ok = true;
#pragma unroll
        for (int x = 0; x < W; x++) ok &= pr[x] == root[x];
        A.verdict[i] = ok ? 0 : -1;
    } else {
        HF::store(A.cur_root + (uint64_t)i * N, root);
    }
}

// One warp owns a contiguous range of `per_warp` (item, chain) tasks.  Every
// lane runs one F step per iteration; a lane whose chain is finished stores
// it and claims the next task of the range (ballot + prefix count), so the
// warp advances at the average chain length rather than the longest one.
template <class HF>
__global__ void k_verify_chains(SetParams P, VerifyArgs A, int L, int per_warp) {
    constexpr int W = HF::W, N = 4 * W, LEN = 2 * N + 3;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t total = (uint64_t)A.count * LEN;
    const uint64_t base = gw * (uint64_t)per_warp;
    if (base >= total) return;
    const uint64_t end = base + per_warp < total ? base + per_warp : total;
    const uint32_t lt_mask = (1u << lane) - 1u;

    bool have = false;
    uint32_t s = 15, item = 0;
    int c = 0;
    uint32_t v[W];
    Adrs wa;
    typename HF::FCtx fc;
    KeyRegs<N> key;
    uint64_t next = base;

    while (true) {
        // retire finished chains and claim new tasks until every lane either
        // has a chain with steps left or the range is exhausted
        while (true) {
            if (have && s >= 15) {
                HF::store(A.wpk + ((uint64_t)item * LEN + c) * N, v);
                have = false;
            }
            const uint32_t need = __ballot_sync(0xffffffffu, !have);
            const uint64_t t = next + __popc(need & lt_mask);
            if (!have && t < end) {
                item = (uint32_t)(t / LEN);
                c = (int)(t % LEN);
                const SignWork wk = A.work[item];
                if (wk.flags) {
                    s = 15;   // rejected item: nothing to compute or store
                    have = false;
                } else {
                    const uint8_t *pkb = A.pk.row(item);
                    key_from_work<HF>(key, pkb, pkb, wk);
                    uint64_t tree_L;
                    uint32_t idx_L;
                    layer_index(P, wk.tree, wk.idx_leaf, L, tree_L, idx_L);
                    uint32_t root[W];
                    HF::load(root, A.cur_root + (uint64_t)item * N);
                    s = chain_len<HF>(P, root, c);
                    adrs_zero(wa);
                    adrs_layer(wa, L);
                    adrs_tree(wa, tree_L);
                    adrs_type(wa, ADDR_WOTS);
                    adrs_keypair(wa, idx_L);
                    adrs_chain(wa, c);
                    HF::f_prepare(fc, wa, key);
                    HF::load(v, A.sig + (uint64_t)item * A.sig_stride + N + P.fors_bytes +
                                    (uint64_t)L * (P.wots_bytes + P.hp * N) + (uint64_t)c * N);
                    have = true;
                }
            }
            next += __popc(need);
            // keep refilling while a lane holds a finished (zero-step) chain,
            // or a lane is idle and the range still has tasks
            const bool again = __any_sync(0xffffffffu, have && s >= 15) ||
                               (__any_sync(0xffffffffu, !have) && next < end);
            if (!again) break;
        }
        if (!__any_sync(0xffffffffu, have)) break;
        if (have) {
            HF::f_step(v, v, fc, s, key);
            s++;
        }
    }
}

}  // namespace cuspx
