// spx_launch.cuh -- launch sequences for one hash family instantiation.
//
// Each translation unit (spx_family_*.cu) instantiates Family<HF> for its
// (hash, n, robust) combinations and registers them in the dispatch table
// that the host engine indexes by parameter set.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "spx_kernels.cuh"
#include "spx_verify.cuh"
#include "spx_vsort.cuh"

namespace cuspx {

// launch mapping knobs (picked per parameter set by the autotuner)
struct Tuning {
    int leaf_block = 128;    // threads per block for k_leaves
    int fors_block = 128;    // threads per block for k_fors_sign (multiple of 32)
    int verify_block = 64;   // threads per block for k_verify_root (and k_verify_ht)
    int tree_warps = 4;      // warps per block for k_trees (upper bound)
    int chains_per_warp = 64;  // (item, chain) tasks per warp in k_verify_chains
    int verify_mode = 0;     // 0 layered kernels, 1 one thread per item over all layers,
                             // 2 persistent hypertree kernel, 3 layered with sorted chains
    int fors_lanes_log2 = 5; // lanes per FORS tree = 2^g (0: lane per tree, 5: warp per tree)
    int tree_mode = 0;       // 0 warp per XMSS tree, 1 lane per tree (subtrees of height <= 4)
    int chain_mode_max = 64; // batches of at most this many items run XMSS leaves chain-parallel
    int verify_slots = 4;    // most items per warp in the persistent verify kernel
    int verify_item_max = 0; // batches of at most this many items verify one item per block
    int verify_claim_min = 1;// persistent verify: free lanes before chains are handed out
    int verify_groups = 4;   // sorted verify: item groups on their own streams (1..8)
    int verify_sorted_min = 0; // batches of at least this many items verify as verify_mode 3 (0: never by size)
    int verify_spec_max = 0;   // batches of at most this many items verify with speculative chains (0: never)
};

struct KeygenArgs {
    uint32_t count;
    uint8_t *sk;       // count x 4n: SK_SEED || SK_PRF || PUB_SEED filled in, ROOT written
    uint8_t *pk;       // count x 2n: written
    uint8_t *leaves;   // count x 2^hp x n scratch
    uint8_t *roots;    // count x n scratch
    uint8_t *ends;     // chain-parallel scratch (count x 2^hp x len x n) or null
    uint32_t ends_cap; // items the chain-parallel scratch holds
};

// Optional per-kernel timing: an event is recorded on the launch stream
// after every kernel of a sequence (event 0 before the first).
struct PhaseTimer {
    static constexpr int kMax = 160;
    cudaEvent_t ev[kMax + 1];
    const char *names[kMax];
    int n = 0;
    void mark(const char *name, cudaStream_t s) {
        if (n < kMax) {
            names[n] = name;
            cudaEventRecord(ev[n + 1], s);
            n++;
        }
    }
};
#define CUSPX_MARK(pt, name, s) \
    do {                        \
        if (pt) (pt)->mark(name, s); \
    } while (0)

// A side stream for the part of a sign sequence that runs beside the rest:
// the FORS trees need only the message digest, and the hypertree leaves and
// trees do not need FORS, so k_fors_sign runs on `side` between `fork`
// (recorded after the message kernels) and `join` (waited before
// k_sign_finish).  Works inside graph capture as a fork/join of the graph.
struct StreamFork {
    cudaStream_t side;
    cudaEvent_t fork, join;
};

// Streams of a verify batch for verify_mode 3: group g > 0 runs on side[g-1]
// between `fork` and join[g-1]; chain[g] orders group g+1's chain kernel of a
// layer after group g's.  Works inside graph capture.
struct VerifyFork {
    static constexpr int kMaxGroups = 8;
    int sides = 0;   // side streams available (groups beyond sides + 1 are not used)
    cudaStream_t side[kMaxGroups - 1] = {};
    cudaEvent_t fork = nullptr, join[kMaxGroups - 1] = {}, chain[kMaxGroups - 1] = {};
};

struct FamilyOps {
    cudaError_t (*configure)();
    // long_msg: messages of at least this many bytes are hashed two warps per
    // 32 messages (SHA-256 sets; 0 or a SHAKE set: one thread each).
    // fk: optional side stream (ignored while per-kernel timing is on).
    void (*sign)(const SetParams &, const SignArgs &, const Tuning &, cudaStream_t, PhaseTimer *, uint64_t long_msg,
                 const StreamFork *fk);
    // vl / vf: bucket lists and streams of verify_mode 3 (null: that mode
    // runs as verify_mode 2)
    void (*verify)(const SetParams &, const VerifyArgs &, const Tuning &, cudaStream_t, PhaseTimer *,
                   uint64_t long_msg, const VerifyLists *vl, const VerifyFork *vf);
    void (*keygen)(const SetParams &, const KeygenArgs &, const Tuning &, cudaStream_t, PhaseTimer *);
    int smem_words;    // per-thread T_l stream scratch
};

// registry: [hash][n index 0..2][robust]
extern FamilyOps g_family[2][3][2];

inline unsigned ceil_div(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

// SM count of the current device, queried once per device (a launch-shape
// input of the small-batch mappings; 1 if the query fails)
inline int device_sms() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        v = sms > 0 ? sms : 1;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

// finish key generation: sk.ROOT = pk.ROOT = top root, pk.PUB_SEED = sk.PUB_SEED
template <int n>
__global__ void k_keygen_finish(KeygenArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.count) return;
    uint8_t *sk = A.sk + (uint64_t)i * 4 * n;
    uint8_t *pk = A.pk + (uint64_t)i * 2 * n;
    for (int j = 0; j < n; j++) {
        const uint8_t r = A.roots[(uint64_t)i * n + j];
        sk[3 * n + j] = r;
        pk[n + j] = r;
        pk[j] = sk[2 * n + j];
    }
}

template <class HF>
struct Family {
    static constexpr int W = HF::W, N = 4 * W;

    static cudaError_t configure() {
        cudaError_t e;
        const int big = 200 * 1024;
        if ((e = cudaFuncSetAttribute(k_leaves<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_leaf_tlen<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_fors_sign<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_trees<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_verify_ht<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_verify_root<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if constexpr (kPersistVerify)
            if ((e = cudaFuncSetAttribute(k_verify_hyper<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big)))
                return e;
        if ((e = cudaFuncSetAttribute(k_verify_item<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_vsort_layer<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_vspec_walk<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        if ((e = cudaFuncSetAttribute(k_sign_finish<HF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
        // Load every other kernel of the family now: with lazy module loading
        // a kernel's first launch loads it, and in a server that first launch
        // is a request's (one took ~50 ms of host time and held back every
        // queued request of its class).
        cudaFuncAttributes fa;
        const void *rest[] = {(const void *)k_sign_msg<HF>, (const void *)k_leaf_chains<HF>,
                              (const void *)k_trees_lane<HF>, (const void *)k_sign_finish<HF>,
                              (const void *)k_verify_msg<HF>, (const void *)k_verify_fors<HF>,
                              (const void *)k_verify_chains<HF>, (const void *)k_vsort_chains<HF>,
                              (const void *)k_vspec_cand<HF>,
                              (const void *)k_keygen_finish<N>};
        for (const void *f : rest)
            if ((e = cudaFuncGetAttributes(&fa, f))) return e;
        if constexpr (!HF::kShake) {
            if ((e = cudaFuncGetAttributes(&fa, (const void *)k_sign_msg_pair<HF>))) return e;
            if ((e = cudaFuncGetAttributes(&fa, (const void *)k_verify_msg_pair<HF>))) return e;
        } else {
            if ((e = cudaFuncGetAttributes(&fa, (const void *)k_sign_msg_wide<HF>))) return e;
            if ((e = cudaFuncGetAttributes(&fa, (const void *)k_verify_msg_wide<HF>))) return e;
        }
        return cudaSuccess;
    }

    // the persistent verify kernel covers every set (the robust SHA-256
    // policy lays its slot out for subtrees of height <= 9, the tallest of
    // any set)
    static constexpr bool kPersistVerify = true;

    // one launch over the batch's whole hypertree: as many blocks as are
    // resident at once (or fewer for small batches); warps take items from
    // the counter as their slots free up
    static void verify_persistent(const SetParams &P, const VerifyArgs &A, const Tuning &tu, cudaStream_t s,
                                  PhaseTimer *pt) {
        if constexpr (kPersistVerify) {
            int wpb = tu.verify_block / 32;
            wpb = wpb < 1 ? 1 : (wpb > 4 ? 4 : wpb);
            const int sms = device_sms();
            int occ = 0;
            // Items per warp: one item's serial critical path (~d x 20
            // compressions) sets the time of a small batch, and a warp
            // holding several items runs their paths at a fraction of its
            // lanes each, so a batch first spreads to about 4 warps per SM
            // and only then packs up to verify_slots items per warp.
            const int gmax = tu.verify_slots < 1 ? 1 : (tu.verify_slots > 8 ? 8 : tu.verify_slots);
            int G = (int)ceil_div(A.count, 4ull * sms);
            G = G < 1 ? 1 : (G > gmax ? gmax : G);
            const size_t smem = (size_t)wpb * G * VerifyPolicy<HF>::slot_words(P.hp) * 4;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_verify_hyper<HF>, 32 * wpb, smem);
            if (occ < 1) occ = 1;
            const uint64_t want = ceil_div(A.count, (uint64_t)G * wpb);
            const uint64_t cap = (uint64_t)occ * (sms > 0 ? sms : 1);
            cudaMemsetAsync(A.ctr, 0, sizeof(uint32_t), s);
            const int claim_min = tu.verify_claim_min < 1 ? 1 : (tu.verify_claim_min > 32 ? 32 : tu.verify_claim_min);
            k_verify_hyper<HF><<<(unsigned)(want < cap ? want : cap), 32 * wpb, smem, s>>>(P, A, A.ctr, G, claim_min);
            CUSPX_MARK(pt, "k_verify_hyper", s);
        }
    }

    static void trees(const SetParams &P, const TreeArgs &T, const Tuning &tu, cudaStream_t s) {
        if (tu.tree_mode == 1 && P.hp <= 4) {
            const uint64_t threads = (uint64_t)T.count * T.nlayers;
            k_trees_lane<HF><<<ceil_div(threads, 128), 128, 0, s>>>(P, T);
            return;
        }
        const uint64_t per_warp = 2ull * (1u << P.hp) * W * 4;
        int wpb = (int)(48 * 1024 / per_warp);
        if (wpb > tu.tree_warps) wpb = tu.tree_warps;
        if (wpb < 1) wpb = 1;
        const uint64_t warps = (uint64_t)T.count * T.nlayers;
        k_trees<HF><<<ceil_div(warps, wpb), 32 * wpb, per_warp * wpb, s>>>(P, T);
    }

    // XMSS leaves: one thread per leaf (k_leaves), or for small batches one
    // thread per chain then one per leaf (k_leaf_chains + k_leaf_tlen)
    static void leaves(const SetParams &P, const LeafArgs &L, const Tuning &tu, cudaStream_t s, PhaseTimer *pt,
                       bool chain_mode) {
        const uint64_t nleaves = (uint64_t)L.count * L.nlayers * (1u << P.hp);
        if (chain_mode) {
            constexpr int LEN = 2 * N + 3;
            k_leaf_chains<HF><<<ceil_div(nleaves * LEN, 128), 128, 0, s>>>(P, L);
            CUSPX_MARK(pt, "k_leaf_chains", s);
            if (L.work) {   // signing: 32 threads per block, each with a slot of 1-5 KB
                const uint32_t sw = VsortSmem<HF>::slot_stride(0);
                k_leaf_tlen<HF><<<ceil_div(nleaves, 32), 32, (size_t)32 * sw * 4, s>>>(P, L, sw);
            } else {
                k_leaf_tlen<HF><<<ceil_div(nleaves, 64), 64, (size_t)64 * HF::kSmemWords * 4, s>>>(P, L, 0u);
            }
            CUSPX_MARK(pt, "k_leaf_tlen", s);
            return;
        }
        const int b = tu.leaf_block;
        k_leaves<HF><<<ceil_div(nleaves, b), b, (size_t)b * HF::kSmemWords * 4, s>>>(P, L);
        CUSPX_MARK(pt, "k_leaves", s);
    }

    static void sign(const SetParams &P, const SignArgs &A, const Tuning &tu, cudaStream_t s, PhaseTimer *pt,
                     uint64_t long_msg, const StreamFork *fk) {
        if (A.count == 0) return;
        k_sign_msg<HF><<<ceil_div(A.count, 128), 128, 0, s>>>(P, A, long_msg);
        CUSPX_MARK(pt, "k_sign_msg", s);
        if (long_msg) {   // messages of >= long_msg bytes: two warps per 32 (SHA-256), a warp each (SHAKE)
            if constexpr (!HF::kShake) {
                k_sign_msg_pair<HF><<<ceil_div(A.count, 32), 64, 0, s>>>(P, A, long_msg);
                CUSPX_MARK(pt, "k_sign_msg_pair", s);
            } else {
                k_sign_msg_wide<HF><<<ceil_div(A.count, 4), 128, 0, s>>>(P, A, long_msg);
                CUSPX_MARK(pt, "k_sign_msg_wide", s);
            }
        }
        const bool split = fk && !pt;
        cudaStream_t sf = split ? fk->side : s;
        if (split) {
            cudaEventRecord(fk->fork, s);
            cudaStreamWaitEvent(sf, fk->fork, 0);
        }
        {
            const int b = tu.fors_block;
            // small batches: spread each tree over more lanes until the launch
            // has about one full wave of threads (SMs x 128), for latency
            const uint64_t wave = (uint64_t)device_sms() * 128;
            int g = tu.fors_lanes_log2 < P.a ? tu.fors_lanes_log2 : P.a;
            while (g < 5 && g < P.a && (((uint64_t)A.count * P.k) << g) < wave) g++;
            const uint64_t threads = (((uint64_t)A.count * P.k) << g);
            k_fors_sign<HF><<<ceil_div(threads, b), b, (size_t)b * (P.a - g + 1) * W * 4, sf>>>(P, A, g);
            CUSPX_MARK(pt, "k_fors_sign", s);
        }
        if (split) cudaEventRecord(fk->join, sf);
        {
            LeafArgs L{A.count, 0, P.d, A.sk, A.work, A.leaves, A.chains, A.ends};
            leaves(P, L, tu, s, pt, A.ends && A.count <= (uint32_t)tu.chain_mode_max && A.count <= A.ends_cap);
        }
        {
            TreeArgs T{A.count, 0, P.d, A.sk, A.work, A.leaves, A.roots, A.sig};
            trees(P, T, tu, s);
            CUSPX_MARK(pt, "k_trees", s);
        }
        if (split) cudaStreamWaitEvent(s, fk->join, 0);
        k_sign_finish<HF><<<A.count, 128, (8 + VsortSmem<HF>::slot_stride(0)) * 4, s>>>(P, A);
        CUSPX_MARK(pt, "k_sign_finish", s);
    }

    static constexpr uint32_t kLayerSmem = 200u * 1024u;   // the shared-memory limit configure() sets

    // verify_mode 3: per group of items, T_k then per layer the sorted
    // chains and the layer roots (spx_vsort.cuh).  Groups run on their own
    // streams; a group's chain kernel of layer L starts after the previous
    // group's, so the groups keep an offset and one group's serial layer
    // kernel overlaps the next group's chains.  With per-kernel timing on
    // every group runs on s.
    static void verify_sorted(const SetParams &P, const VerifyArgs &A, const Tuning &tu, cudaStream_t s,
                              PhaseTimer *pt, const VerifyLists &V, const VerifyFork *vf) {
        constexpr int LEN = 2 * N + 3;
        int G = tu.verify_groups < 1 ? 1 : tu.verify_groups;
        const int gmax = pt || !vf ? 1 : vf->sides + 1;
        if (G > gmax) G = gmax;
        if ((uint32_t)G > A.count) G = (int)A.count;
        const uint32_t per = (A.count + G - 1) / G;
        G = (int)((A.count + per - 1) / per);
        // thread per item in the layer kernel, whose slots must fit the
        // 200 KiB of shared memory configured for it (32 threads fit for
        // every set: SHAKE-256f-robust needs 176 KiB)
        int b = tu.verify_block;
        while (b > 32 && VsortSmem<HF>::bytes(P, (uint32_t)b) > kLayerSmem) b /= 2;
        const size_t smem = VsortSmem<HF>::bytes(P, (uint32_t)b);
        cudaMemsetAsync(V.cnt, 0, (size_t)G * P.d * 16 * sizeof(uint32_t), s);
        cudaStream_t gs[VerifyFork::kMaxGroups];
        gs[0] = s;
        if (G > 1) cudaEventRecord(vf->fork, s);
        for (int g = 1; g < G; g++) {
            gs[g] = vf->side[g - 1];
            cudaStreamWaitEvent(gs[g], vf->fork, 0);
        }
        auto first = [&](int g) { return (uint32_t)g * per; };
        auto items = [&](int g) { return g + 1 < G ? per : A.count - (uint32_t)g * per; };
        for (int g = 0; g < G; g++) {
            k_verify_fors<HF><<<ceil_div((uint64_t)items(g) * P.k, 128), 128, 0, gs[g]>>>(P, A, first(g), items(g));
            CUSPX_MARK(pt, "k_verify_fors", s);
            k_vsort_layer<HF><<<ceil_div(items(g), b), b, smem, gs[g]>>>(P, A, V, -1, first(g), items(g), g);
            CUSPX_MARK(pt, "k_vsort_layer", s);
        }
        for (int L = 0; L < P.d; L++) {
            for (int g = 0; g < G; g++) {
                if (g > 0) cudaStreamWaitEvent(gs[g], vf->chain[g - 1], 0);
                k_vsort_chains<HF><<<ceil_div((uint64_t)items(g) * LEN, 128), 128, 0, gs[g]>>>(P, A, V, L, first(g), g);
                CUSPX_MARK(pt, "k_vsort_chains", s);
                if (g + 1 < G) cudaEventRecord(vf->chain[g], gs[g]);
                k_vsort_layer<HF><<<ceil_div(items(g), b), b, smem, gs[g]>>>(P, A, V, L, first(g), items(g), g);
                CUSPX_MARK(pt, "k_vsort_layer", s);
            }
        }
        for (int g = 1; g < G; g++) {
            cudaEventRecord(vf->join[g - 1], gs[g]);
            cudaStreamWaitEvent(s, vf->join[g - 1], 0);
        }
    }

    static void verify(const SetParams &P, const VerifyArgs &A, const Tuning &tu, cudaStream_t s, PhaseTimer *pt,
                       uint64_t long_msg, const VerifyLists *vl, const VerifyFork *vf) {
        if (A.count == 0) return;
        k_verify_msg<HF><<<ceil_div(A.count, 128), 128, 0, s>>>(P, A, long_msg);
        CUSPX_MARK(pt, "k_verify_msg", s);
        if (long_msg) {
            if constexpr (!HF::kShake) {
                k_verify_msg_pair<HF><<<ceil_div(A.count, 32), 64, 0, s>>>(P, A, long_msg);
                CUSPX_MARK(pt, "k_verify_msg_pair", s);
            } else {
                k_verify_msg_wide<HF><<<ceil_div(A.count, 4), 128, 0, s>>>(P, A, long_msg);
                CUSPX_MARK(pt, "k_verify_msg_wide", s);
            }
        }
        const bool want_sorted =
            tu.verify_mode == 3 || (tu.verify_sorted_min > 0 && A.count >= (uint32_t)tu.verify_sorted_min);
        const bool sorted = want_sorted && vl && vl->tasks && vl->stride >= (uint64_t)A.count * (2 * N + 3) &&
                            A.count < (1u << 25) && VsortSmem<HF>::bytes(P, 32) <= kLayerSmem && P.len1 == 2 * N &&
                            P.len2 == 3 && !(tu.verify_item_max > 0 && A.count <= (uint32_t)tu.verify_item_max);
        if (sorted) {   // FORS per item group, beside the other groups' layers
            verify_sorted(P, A, tu, s, pt, *vl, vf);
            return;
        }
        if (tu.verify_spec_max > 0 && A.count <= (uint32_t)tu.verify_spec_max && vl && vl->cand &&
            A.count <= vl->cand_items && 32u * VsortSmem<HF>::slot_stride(P.hp) * 4u <= kLayerSmem &&
            P.len1 == 2 * N && P.len2 == 3) {
            // tiny batches: every chain run from every start step, then the
            // serial walk over T_len and the auth paths alone (spx_vsort.cuh)
            // (the chain runs beside the FORS roots, on a side stream)
            constexpr int LEN = 2 * N + 3;
            const bool side = !pt && vf && vf->sides > 0;
            cudaStream_t cs = side ? vf->side[0] : s;
            if (side) {
                cudaEventRecord(vf->fork, s);
                cudaStreamWaitEvent(cs, vf->fork, 0);
            }
            k_vspec_cand<HF><<<ceil_div(16ull * A.count * P.d * LEN, 128), 128, 0, cs>>>(P, A, vl->cand);
            CUSPX_MARK(pt, "k_vspec_cand", s);
            k_verify_fors<HF><<<ceil_div((uint64_t)A.count * P.k, 128), 128, 0, s>>>(P, A, 0, A.count);
            CUSPX_MARK(pt, "k_verify_fors", s);
            if (side) {
                cudaEventRecord(vf->join[0], cs);
                cudaStreamWaitEvent(s, vf->join[0], 0);
            }
            k_vspec_walk<HF><<<ceil_div(A.count, 32), 32, 32u * VsortSmem<HF>::slot_stride(P.hp) * 4u, s>>>(
                P, A, vl->cand);
            CUSPX_MARK(pt, "k_vspec_walk", s);
            return;
        }
        k_verify_fors<HF><<<ceil_div((uint64_t)A.count * P.k, 128), 128, 0, s>>>(P, A, 0, A.count);
        CUSPX_MARK(pt, "k_verify_fors", s);
        if (tu.verify_item_max > 0 && A.count <= (uint32_t)tu.verify_item_max && P.hp <= 9) {
            // small batches: one item per block (its serial path sets the time)
            constexpr int LEN = 2 * N + 3, CW = (LEN + 31) / 32;
            // one slot and the prefetched auth path of the next layer
            const size_t smem = ((size_t)VerifyPolicy<HF>::slot_words(P.hp) + (size_t)P.hp * W) * 4;
            k_verify_item<HF><<<A.count, 32 * (CW + 1), smem, s>>>(P, A);
            CUSPX_MARK(pt, "k_verify_item", s);
            return;
        }
        const int b = tu.verify_block;
        if (tu.verify_mode >= 2 && kPersistVerify && A.ctr && P.hp <= 9) {
            verify_persistent(P, A, tu, s, pt);
            return;
        }
        if (tu.verify_mode == 1) {
            k_verify_ht<HF><<<ceil_div(A.count, b), b, (size_t)b * HF::kSmemWords * 4, s>>>(P, A);
            CUSPX_MARK(pt, "k_verify_ht", s);
            return;
        }
        constexpr int LEN = 2 * N + 3;
        const int pw = tu.chains_per_warp;
        const uint64_t warps = ((uint64_t)A.count * LEN + pw - 1) / pw;
        for (int L = -1; L < P.d; L++) {
            if (L >= 0) {
                k_verify_chains<HF><<<ceil_div(warps, 4), 128, 0, s>>>(P, A, L, pw);
                CUSPX_MARK(pt, "k_verify_chains", s);
            }
            k_verify_root<HF><<<ceil_div(A.count, b), b, (size_t)b * HF::kSmemWords * 4, s>>>(P, A, L);
            CUSPX_MARK(pt, "k_verify_root", s);
        }
    }

    static void keygen(const SetParams &P, const KeygenArgs &K, const Tuning &tu, cudaStream_t s, PhaseTimer *pt) {
        if (K.count == 0) return;
        KeyRef kr{K.sk, nullptr, (uint32_t)(4 * N)};
        LeafArgs L{K.count, P.d - 1, 1, kr, nullptr, K.leaves, nullptr, K.ends};
        // the top layer alone is 2^hp leaves per key, so one lane per leaf
        // leaves SMs idle up to thousands of keys (4096 keys: 1.27 ms one
        // lane per leaf, 1.17 ms one lane per chain); chain lanes whenever
        // the scratch holds the batch, unless chain_mode_max is 0
        leaves(P, L, tu, s, pt, K.ends && tu.chain_mode_max > 0 && K.count <= K.ends_cap);
        TreeArgs T{K.count, P.d - 1, 1, kr, nullptr, K.leaves, K.roots, nullptr};
        trees(P, T, tu, s);
        CUSPX_MARK(pt, "k_trees", s);
        k_keygen_finish<N><<<ceil_div(K.count, 128), 128, 0, s>>>(K);
        CUSPX_MARK(pt, "k_keygen_finish", s);
    }

    static FamilyOps ops() {
        FamilyOps o;
        o.configure = &configure;
        o.sign = &sign;
        o.verify = &verify;
        o.keygen = &keygen;
        o.smem_words = HF::kSmemWords;
        return o;
    }
};

}  // namespace cuspx
