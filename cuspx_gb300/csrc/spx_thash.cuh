// spx_thash.cuh -- SPHINCS+ tweakable hash families on top of spx_hash.cuh.
//
// Two policy classes with one interface, instantiated per (n, robust):
//   Sha2<N, ROBUST>   thash_sha256.cu:16-34 (simple), hash_sha256.cu:65-326
//   Shake<N, ROBUST>  thash_shake256.cu:15-25 (simple), hash_shake256.cu:38-130
// Robust thash is not in the reference; it follows the published SPHINCS+
// round-3 robust construction: the input is xored with a bitmask drawn from
// MGF1-SHA256(PUB_SEED || ADRS_c) or SHAKE256(PUB_SEED || ADRS).
//
//   F(out, in, adrs, key)        one n-byte block
//   H(out, l, r, adrs, key)      two n-byte blocks
//   PRF(out, adrs, key)          secret chain/leaf start value
//   TStream                      T_l over a stream of n-byte values (T_len,
//                                T_k), absorbing as values are produced
//   prf_msg / h_msg              message randomiser and message digest over
//                                a message in global memory
#pragma once
#include "spx_hash.cuh"

#ifndef CUSPX_ROBUST_LEAF_MINBLOCKS
#define CUSPX_ROBUST_LEAF_MINBLOCKS 1
#endif

namespace cuspx {

// Per-item key material in registers.  mid is the SHA-256 state after the
// 64-byte block PUB_SEED || 0^(64-n) (the reference's process-global
// state_seeded, sha256.cu:385-405, here one per key).
template <int N>
struct KeyRegs {
    static constexpr int W = N / 4;
    uint32_t pub[W];
    uint32_t skseed[W];
    uint32_t mid[8];
};

// ---------------------------------------------------------------------------
// global-memory helpers for n-byte strings (all offsets multiples of 8)
// ---------------------------------------------------------------------------
template <int N>
SPX_DEV void load_bytes_le(uint32_t v[N / 4], const uint8_t *p) {
    if (N % 16 == 0 && ((uintptr_t)p & 15) == 0) {
#pragma unroll
        for (int i = 0; i < N / 16; i++) {
            uint4 q = reinterpret_cast<const uint4 *>(p)[i];
            v[4 * i] = q.x; v[4 * i + 1] = q.y; v[4 * i + 2] = q.z; v[4 * i + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N / 8; i++) {
            uint2 q = reinterpret_cast<const uint2 *>(p)[i];
            v[2 * i] = q.x; v[2 * i + 1] = q.y;
        }
    }
}
template <int N>
SPX_DEV void store_bytes_le(uint8_t *p, const uint32_t v[N / 4]) {
    if (N % 16 == 0 && ((uintptr_t)p & 15) == 0) {
#pragma unroll
        for (int i = 0; i < N / 16; i++)
            reinterpret_cast<uint4 *>(p)[i] = make_uint4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < N / 8; i++) reinterpret_cast<uint2 *>(p)[i] = make_uint2(v[2 * i], v[2 * i + 1]);
    }
}

// ===========================================================================
// SHA-256 family
// ===========================================================================
template <int N, bool ROBUST>
struct Sha2 {
    static constexpr int W = N / 4;
    static constexpr bool kRobust = ROBUST;
    static constexpr int kShake = 0;
    // k_leaves occupancy floor for robust chains (which carry a second, mask
    // state); measured on GB300, capping registers to raise it spills and is
    // slower, so the default leaves the compiler's choice
    static constexpr int kLeafMinBlocks = ROBUST ? CUSPX_ROBUST_LEAF_MINBLOCKS : 1;

    // memory <-> register order
    SPX_DEV static void load(uint32_t v[W], const uint8_t *p) {
        load_bytes_le<N>(v, p);
#pragma unroll
        for (int i = 0; i < W; i++) v[i] = bswap32(v[i]);
    }
    SPX_DEV static void store(uint8_t *p, const uint32_t v[W]) {
        uint32_t t[W];
#pragma unroll
        for (int i = 0; i < W; i++) t[i] = bswap32(v[i]);
        store_bytes_le<N>(p, t);
    }

    // midstate after PUB_SEED || 0^(64-n)  (seed_state, sha256.cu:391-405)
    SPX_DEV static void key_init(KeyRegs<N> &k, const uint8_t *skseed, const uint8_t *pub) {
        load(k.skseed, skseed);
        load(k.pub, pub);
        uint32_t w[16];
#pragma unroll
        for (int i = 0; i < 16; i++) w[i] = i < W ? k.pub[i] : 0u;
        sha256_iv(k.mid);
        sha256_compress(k.mid, w);
    }

    // SHA256(midstate; ADRS_c || in[L words]), truncated (thash_sha256.cu:16-34)
    template <int L>
    SPX_DEV static void core(uint32_t out[W], const uint32_t mid[8], const Adrs &a, const uint32_t in[L]) {
        constexpr int TOT = 22 + 4 * L;
        constexpr int NB = (TOT + 9 + 63) / 64;
        uint32_t m[16 * NB];
#pragma unroll
        for (int i = 0; i < 5; i++) m[i] = a.w[i];
        m[5] = (a.w[5] & 0xffff0000u) | (in[0] >> 16);
#pragma unroll
        for (int i = 1; i < L; i++) m[5 + i] = __funnelshift_l(in[i], in[i - 1], 16);
        m[5 + L] = (in[L - 1] << 16) | 0x8000u;
#pragma unroll
        for (int i = 6 + L; i < 16 * NB; i++) m[i] = 0;
        m[16 * NB - 1] = (64 + TOT) * 8;
        uint32_t s[8];
#pragma unroll
        for (int i = 0; i < 8; i++) s[i] = mid[i];
        sha256_compress(s, m);
        if (NB == 2) sha256_compress(s, m + 16);
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = s[i];
    }

    // MGF1-SHA256(PUB_SEED || ADRS_c, .) block `ctr` (sha256.cu:362-383)
    SPX_DEV static void mask_block(uint32_t out[8], const uint32_t pub[W], const Adrs &a, uint32_t ctr) {
        constexpr int TOT = N + 26;
        constexpr int NB = (TOT + 9 + 63) / 64;
        uint32_t m[16 * NB];
#pragma unroll
        for (int i = 0; i < W; i++) m[i] = pub[i];
#pragma unroll
        for (int i = 0; i < 5; i++) m[W + i] = a.w[i];
        m[W + 5] = (a.w[5] & 0xffff0000u) | (ctr >> 16);
        m[W + 6] = (ctr << 16) | 0x8000u;
#pragma unroll
        for (int i = W + 7; i < 16 * NB; i++) m[i] = 0;
        m[16 * NB - 1] = TOT * 8;
        sha256_iv(out);
        sha256_compress(out, m);
        if (NB == 2) sha256_compress(out, m + 16);
    }

    template <int L>
    SPX_DEV static void thash(uint32_t out[W], const KeyRegs<N> &k, const Adrs &a, uint32_t in[L]) {
        if (ROBUST) {
#pragma unroll
            for (int b = 0; b < (L + 7) / 8; b++) {
                uint32_t mk[8];
                mask_block(mk, k.pub, a, b);
#pragma unroll
                for (int i = 0; i < 8; i++)
                    if (8 * b + i < L) in[8 * b + i] ^= mk[i];
            }
        }
        core<L>(out, k.mid, a, in);
    }

    SPX_DEV static void F(uint32_t out[W], const uint32_t in[W], const Adrs &a, const KeyRegs<N> &k) {
        uint32_t t[W];
#pragma unroll
        for (int i = 0; i < W; i++) t[i] = in[i];
        thash<W>(out, k, a, t);
    }
    SPX_DEV static void H(uint32_t out[W], const uint32_t l[W], const uint32_t r[W], const Adrs &a,
                          const KeyRegs<N> &k) {
        uint32_t t[2 * W];
#pragma unroll
        for (int i = 0; i < W; i++) { t[i] = l[i]; t[W + i] = r[i]; }
        thash<2 * W>(out, k, a, t);
    }

    // ---- WOTS+ chain steps ------------------------------------------------
    // Along one chain the ADRS differs only in its hash byte (byte 21, in
    // message word 5), so rounds 0..4 of every F compression -- and rounds
    // 0..W+4 of the robust mask compression -- are the same for all steps.
    // f_prepare runs them once; f_step starts each compression after them.
    struct FCtx {
        uint32_t st[8];     // state after rounds 0..4 from the midstate
        uint32_t m[5];      // ADRS words 0..4
        uint32_t a5;        // ADRS word 5 without the hash byte
        uint32_t mst[ROBUST ? 8 : 1];   // robust: mask state after rounds 0..W+4 from the IV
    };
    SPX_DEV static void f_prepare(FCtx &f, const Adrs &a, const KeyRegs<N> &k) {
        uint32_t w[16];
#pragma unroll
        for (int i = 0; i < 5; i++) f.m[i] = w[i] = a.w[i];
        f.a5 = a.w[5] & 0xff000000u;
#pragma unroll
        for (int i = 0; i < 8; i++) f.st[i] = k.mid[i];
        sha256_rounds<0, 5>(f.st, w);
        if (ROBUST) {
            uint32_t x[16];
#pragma unroll
            for (int i = 0; i < W; i++) x[i] = k.pub[i];
#pragma unroll
            for (int i = 0; i < 5; i++) x[W + i] = a.w[i];
            sha256_iv(f.mst);
            sha256_rounds<0, W + 5>(f.mst, x);
        }
    }
    // out = F(in) at hash address `hash` of the prepared chain
    SPX_DEV static void f_step(uint32_t out[W], const uint32_t in[W], const FCtx &f, uint32_t hash,
                               const KeyRegs<N> &k) {
        const uint32_t a5 = f.a5 | (hash << 16);
        uint32_t x[W];
#pragma unroll
        for (int i = 0; i < W; i++) x[i] = in[i];
        if (ROBUST) {
            // bitmask block 0 = SHA256(PUB_SEED || ADRS_c || BE32(0)), resumed after the prefix
            constexpr int TOT = N + 26;
            constexpr int NB = (TOT + 9 + 63) / 64;
            uint32_t mw[16 * NB];
#pragma unroll
            for (int i = 0; i < W; i++) mw[i] = k.pub[i];
#pragma unroll
            for (int i = 0; i < 5; i++) mw[W + i] = f.m[i];
            mw[W + 5] = a5;
            mw[W + 6] = 0x8000u;
#pragma unroll
            for (int i = W + 7; i < 16 * NB; i++) mw[i] = 0;
            mw[16 * NB - 1] = TOT * 8;
            uint32_t t[8], ms[8];
#pragma unroll
            for (int i = 0; i < 8; i++) t[i] = f.mst[i];
            sha256_rounds<W + 5, 64>(t, mw);
#pragma unroll
            for (int i = 0; i < 8; i++) ms[i] = t[i] + sha256_iv_word(i);
            if (NB == 2) sha256_compress(ms, mw + 16);
#pragma unroll
            for (int i = 0; i < W; i++) x[i] ^= ms[i];
        }
        constexpr int TOT = 22 + N;   // always one block for n <= 32
        uint32_t m[16];
#pragma unroll
        for (int i = 0; i < 5; i++) m[i] = f.m[i];
        m[5] = a5 | (x[0] >> 16);
#pragma unroll
        for (int i = 1; i < W; i++) m[5 + i] = __funnelshift_l(x[i], x[i - 1], 16);
        m[5 + W] = (x[W - 1] << 16) | 0x8000u;
#pragma unroll
        for (int i = 6 + W; i < 16; i++) m[i] = 0;
        m[15] = (64 + TOT) * 8;
        uint32_t t[8];
#pragma unroll
        for (int i = 0; i < 8; i++) t[i] = f.st[i];
        sha256_rounds<5, 64>(t, m);
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = t[i] + k.mid[i];
    }

    // PRF = SHA256(SK_SEED || ADRS_c), no midstate (hash_sha256.cu:65-77)
    SPX_DEV static void PRF(uint32_t out[W], const Adrs &a, const KeyRegs<N> &k) {
        uint32_t m[16];
#pragma unroll
        for (int i = 0; i < W; i++) m[i] = k.skseed[i];
#pragma unroll
        for (int i = 0; i < 5; i++) m[W + i] = a.w[i];
        m[W + 5] = (a.w[5] & 0xffff0000u) | 0x8000u;
#pragma unroll
        for (int i = W + 6; i < 16; i++) m[i] = 0;
        m[15] = (N + 22) * 8;
        uint32_t s[8];
        sha256_iv(s);
        sha256_compress(s, m);
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = s[i];
    }

    // T_l streaming: midstate; ADRS_c || v_0 || v_1 ... Every value lands at a
    // byte offset that is 2 mod 4, so each word straddles two buffer words.
    // buf is a per-thread shared-memory area of kSmemWords words.
    static constexpr int kSmemWords = 17 + (ROBUST ? 8 : 0);
    struct TStream {
        uint32_t st[8];
        uint32_t *buf;
        int pos;        // byte position in the current block, == 2 mod 4
        uint32_t q;     // data words absorbed (for the robust mask)
        uint32_t blocks;
        Adrs a;
    };
    SPX_DEV static void t_init(TStream &t, uint32_t *smem, const KeyRegs<N> &k, const Adrs &a) {
        t.buf = smem;
#pragma unroll
        for (int i = 0; i < 8; i++) t.st[i] = k.mid[i];
#pragma unroll
        for (int i = 0; i < 5; i++) t.buf[i] = a.w[i];
        t.buf[5] = a.w[5] & 0xffff0000u;
        t.pos = 22;
        t.q = 0;
        t.blocks = 0;
        t.a = a;
    }
    SPX_DEV static void t_flush(TStream &t) {
        uint32_t w[16];
#pragma unroll
        for (int i = 0; i < 16; i++) w[i] = t.buf[i];
        sha256_compress(t.st, w);
        t.blocks++;
    }
    SPX_DEV static void t_word(TStream &t, uint32_t x, const KeyRegs<N> &k) {
        if (ROBUST) {
            uint32_t *mb = t.buf + 17;
            if ((t.q & 7) == 0) {
                uint32_t mk[8];
                mask_block(mk, k.pub, t.a, t.q >> 3);
#pragma unroll
                for (int i = 0; i < 8; i++) mb[i] = mk[i];
            }
            x ^= mb[t.q & 7];
        }
        t.q++;
        int wi = t.pos >> 2;
        t.buf[wi] |= x >> 16;
        t.buf[wi + 1] = x << 16;
        t.pos += 4;
        if (t.pos > 64) {
            t_flush(t);
            t.buf[0] = t.buf[16];
            t.pos -= 64;
        }
    }
    SPX_DEV static void t_absorb(TStream &t, const uint32_t v[W], const KeyRegs<N> &k) {
#pragma unroll
        for (int i = 0; i < W; i++) t_word(t, v[i], k);
    }
    SPX_DEV static void t_final(uint32_t out[W], TStream &t) {
        uint32_t bits = (uint32_t)(64 + 64 * t.blocks + t.pos) * 8u;
        int wi = t.pos >> 2;
        t.buf[wi] |= 0x8000u;
        for (int i = wi + 1; i < 16; i++) t.buf[i] = 0;
        if (t.pos + 1 > 56) {
            t_flush(t);
            for (int i = 0; i < 16; i++) t.buf[i] = 0;
        }
        t.buf[15] = bits;
        t_flush(t);
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = t.st[i];
    }

    // ---- message hashing over a message in global memory -----------------
    // word q (big-endian) of the padded stream "prefix(P words) || m || 0x80
    // || 0* || bitlen64"; m must be 4-byte aligned and readable up to the
    // next multiple of 4 bytes.
    SPX_DEV static uint32_t msg_word(const uint8_t *m, uint64_t mlen, uint64_t q) {
        uint64_t b = 4 * q;
        if (b + 4 <= mlen) return bswap32(*reinterpret_cast<const uint32_t *>(m + b));
        if (b > mlen) return 0;
        uint32_t keep = (uint32_t)(mlen - b);  // 0..3 message bytes in this word
        uint32_t x = keep ? bswap32(*reinterpret_cast<const uint32_t *>(m + b)) : 0u;
        uint32_t hi = keep ? (0xffffffffu << (32 - 8 * keep)) : 0u;
        return (x & hi) | (0x80u << (24 - 8 * keep));
    }
    // 16 big-endian message words starting at word q0, all inside m; the
    // word offset keeps the alignment the prefix length gives (P % 4 == 0:
    // 16-byte, P even: 8-byte, else 4-byte) since m itself is 16-byte aligned
    template <int P>
    SPX_DEV static void msg_block_full(uint32_t w[16], const uint8_t *m, uint64_t q0) {
        const uint8_t *p = m + 4 * q0;
        if (P % 4 == 0) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const uint4 v = reinterpret_cast<const uint4 *>(p)[i];
                w[4 * i] = bswap32(v.x); w[4 * i + 1] = bswap32(v.y);
                w[4 * i + 2] = bswap32(v.z); w[4 * i + 3] = bswap32(v.w);
            }
        } else if (P % 2 == 0) {
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const uint2 v = reinterpret_cast<const uint2 *>(p)[i];
                w[2 * i] = bswap32(v.x); w[2 * i + 1] = bswap32(v.y);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; i++) w[i] = bswap32(reinterpret_cast<const uint32_t *>(p)[i]);
        }
    }
    // Block b of prefix (P words, registers) || m || SHA-256 padding, where
    // bits is the total message length in bits.  Blocks wholly inside the
    // message come from the one-block-ahead vector load in nxt (have), and
    // block b + 1 is loaded into nxt here when it is such a block.
    template <int P>
    SPX_DEV static void next_block(uint32_t w[16], uint64_t b, uint64_t nblocks, uint64_t bits, const uint32_t pre[P],
                                   const uint8_t *m, uint64_t mlen, uint32_t nxt[16], bool &have) {
        constexpr int PB = (P + 15) / 16;  // blocks that contain prefix words
        auto full = [&](uint64_t x) { return x >= (uint64_t)PB && 4 * (16 * x - P + 16) <= mlen; };
        if (have) {
#pragma unroll
            for (int j = 0; j < 16; j++) w[j] = nxt[j];
        } else if (b < PB) {
#pragma unroll
            for (int pb = 0; pb < PB; pb++) {
                if (pb == (int)b) {
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        const int g = 16 * pb + j;
                        w[j] = g < P ? pre[g < P ? g : 0] : msg_word(m, mlen, (uint64_t)(g - P));
                    }
                }
            }
        } else {
            const uint64_t q0 = 16 * b - P;
#pragma unroll
            for (int j = 0; j < 16; j++) w[j] = msg_word(m, mlen, q0 + j);
        }
        have = b + 1 < nblocks && full(b + 1);
        if (have) msg_block_full<P>(nxt, m, 16 * (b + 1) - P);
        if (b == nblocks - 1) {
            w[14] = (uint32_t)(bits >> 32);
            w[15] = (uint32_t)bits;
        }
    }

    // absorb prefix (P words, registers) || m into st, which has already
    // absorbed pre_blocks 64-byte blocks; out = final state.
    template <int P>
    SPX_DEV static void stream_msg(uint32_t st[8], uint32_t pre_blocks, const uint32_t pre[P], const uint8_t *m,
                                   uint64_t mlen) {
        const uint64_t dbytes = 4 * (uint64_t)P + mlen;
        const uint64_t nblocks = (dbytes + 9 + 63) / 64;
        const uint64_t bits = (64 * (uint64_t)pre_blocks + dbytes) * 8;
        uint32_t nxt[16];
        bool have = false;
        for (uint64_t b = 0; b < nblocks; b++) {
            uint32_t w[16];
            next_block<P>(w, b, nblocks, bits, pre, m, mlen, nxt, have);
            sha256_compress(st, w);
        }
    }

    // The same absorption split over the two warps of a 64-thread block that
    // hashes 32 messages, for long messages: a thread hashing alone is bound
    // by its own instruction issue, about 1.3k ALU instructions per block.
    // For message l, lane l of warp 0 (role 0) builds each block and its
    // schedule with the round constants added into kw, and lane l of warp 1
    // (role 1) runs the 64 rounds from kw a block behind; one __syncthreads
    // per block hands a buffer over.  kw is a shared 2 x 64 x 32-word double
    // buffer with the 32 messages interleaved (kw[(buf * 64 + t) * 32 + l]).
    // Every thread of the block calls this; max_blocks (the same for the
    // whole block) bounds the loop, and threads whose message has fewer
    // blocks, or role 2, only take part in the barriers.  The result is in
    // role 1's st.
    template <int P>
    SPX_DEV static void stream_msg_pair(uint32_t st[8], uint32_t pre_blocks, const uint32_t pre[P],
                                        const uint8_t *m, uint64_t mlen, uint32_t *kw, int role,
                                        uint64_t max_blocks) {
        const uint64_t dbytes = 4 * (uint64_t)P + mlen;
        const uint64_t nblocks = (dbytes + 9 + 63) / 64;
        const uint64_t bits = (64 * (uint64_t)pre_blocks + dbytes) * 8;
        uint32_t *mine = kw + (threadIdx.x & 31);
        uint32_t nxt[16];
        bool have = false;
        for (uint64_t b = 0; b <= max_blocks; b++) {
            if (role == 0 && b < nblocks) {
                uint32_t w[16];
                next_block<P>(w, b, nblocks, bits, pre, m, mlen, nxt, have);
                sha256_schedule_kw<32>(mine + 64 * 32 * (b & 1), w);
            }
            if (role == 1 && b >= 1 && b <= nblocks) sha256_compress_kw<32>(st, mine + 64 * 32 * ((b - 1) & 1));
            __syncthreads();
        }
    }
    // blocks of prefix (P words) || m with SHA-256 padding
    template <int P>
    SPX_DEV static uint64_t msg_blocks(uint64_t mlen) { return (4 * (uint64_t)P + mlen + 9 + 63) / 64; }

    // PRF_msg = HMAC-SHA256(SK_PRF, optrand || m), truncated (hash_sha256.cu:99-145):
    // the inner hash starts from the key block xor ipad, the outer one hashes
    // the key block xor opad and the inner digest
    SPX_DEV static void hmac_start(uint32_t st[8], const uint32_t skprf[W]) {
        uint32_t w[16];
        sha256_iv(st);
#pragma unroll
        for (int i = 0; i < 16; i++) w[i] = (i < W ? skprf[i] : 0u) ^ 0x36363636u;
        sha256_compress(st, w);
    }
    SPX_DEV static void hmac_finish(uint32_t R[W], const uint32_t inner[8], const uint32_t skprf[W]) {
        uint32_t st[8], w[16];
        sha256_iv(st);
#pragma unroll
        for (int i = 0; i < 16; i++) w[i] = (i < W ? skprf[i] : 0u) ^ 0x5c5c5c5cu;
        sha256_compress(st, w);
#pragma unroll
        for (int i = 0; i < 8; i++) w[i] = inner[i];
        w[8] = 0x80000000u;
#pragma unroll
        for (int i = 9; i < 15; i++) w[i] = 0;
        w[15] = (64 + 32) * 8;
        sha256_compress(st, w);
#pragma unroll
        for (int i = 0; i < W; i++) R[i] = st[i];
    }
    SPX_DEV static void prf_msg(uint32_t R[W], const uint32_t skprf[W], const uint32_t optrand[W],
                                const uint8_t *m, uint64_t mlen) {
        uint32_t st[8];
        hmac_start(st, skprf);
        stream_msg<W>(st, 1, optrand, m, mlen);
        hmac_finish(R, st, skprf);
    }

    // PRF_msg (when with_prf; otherwise R is given) and H_msg of one message
    // through a single compression call site: the HMAC ipad block, optrand
    // || m, the opad block, the inner digest, R || PK || m and the MGF1
    // counter blocks run as one sequence of blocks.  With a call site per
    // step (prf_msg + h_msg) a thread hashing alone on its SM runs a fresh
    // ~20 KB copy of the unrolled rounds at every step and waits on
    // instruction fetch; here one copy stays in the instruction cache.
    // dg: dgst_bytes digest bytes (a byte array in registers/local).
    SPX_DEV static void msg_digests(uint32_t R[W], bool with_prf, const uint32_t skprf[W],
                                    const uint32_t optrand[W], const uint32_t pk[2 * W], const uint8_t *m,
                                    uint64_t mlen, uint8_t *dg, int dgst_bytes) {
        const uint64_t nb1 = (4ull * W + mlen + 9 + 63) / 64;   // optrand || m, after the ipad block
        const uint64_t bits1 = (64 + 4ull * W + mlen) * 8;
        const uint64_t nb2 = (12ull * W + mlen + 9 + 63) / 64;  // R || PK || m
        const uint64_t bits2 = (12ull * W + mlen) * 8;
        const uint64_t nm = (uint64_t)(dgst_bytes + 31) / 32;   // MGF1 blocks
        uint32_t st[8], keep[8], pre[3 * W], nxt[16];
        bool have = false;
        int phase = with_prf ? 0 : 4;   // 0 ipad, 1 optrand || m, 2 opad, 3 inner digest, 4 R || PK || m, 5 MGF1
        uint64_t b = 0;
#pragma unroll
        for (int i = 0; i < W; i++) {
            pre[i] = with_prf ? 0u : R[i];   // with_prf: R comes from phase 3
            pre[W + i] = pk[i];
            pre[2 * W + i] = pk[W + i];
        }
        sha256_iv(st);
        for (;;) {
            uint32_t w[16];
            if (phase == 0 || phase == 2) {
                const uint32_t pad = phase == 0 ? 0x36363636u : 0x5c5c5c5cu;
#pragma unroll
                for (int i = 0; i < 16; i++) w[i] = (i < W ? skprf[i] : 0u) ^ pad;
            } else if (phase == 1) {
                next_block<W>(w, b, nb1, bits1, optrand, m, mlen, nxt, have);
            } else if (phase == 4) {
                next_block<3 * W>(w, b, nb2, bits2, pre, m, mlen, nxt, have);
            } else {
                // 3: inner digest || padding (64 + 32 bytes); 5: seed || BE32(b) || padding (36 bytes)
#pragma unroll
                for (int i = 0; i < 8; i++) w[i] = keep[i];
                w[8] = phase == 3 ? 0x80000000u : (uint32_t)b;
                w[9] = phase == 3 ? 0u : 0x80000000u;
#pragma unroll
                for (int i = 10; i < 15; i++) w[i] = 0;
                w[15] = phase == 3 ? (64 + 32) * 8 : 36 * 8;
            }
            sha256_compress(st, w);
            if (phase == 0) {
                phase = 1;
                b = 0;
                have = false;
            } else if (phase == 1) {
                if (++b == nb1) {
#pragma unroll
                    for (int i = 0; i < 8; i++) keep[i] = st[i];
                    sha256_iv(st);
                    phase = 2;
                }
            } else if (phase == 2) {
                phase = 3;
            } else if (phase == 3) {
#pragma unroll
                for (int i = 0; i < W; i++) R[i] = pre[i] = st[i];
                sha256_iv(st);
                phase = 4;
                b = 0;
                have = false;
            } else if (phase == 4) {
                if (++b == nb2) {
#pragma unroll
                    for (int i = 0; i < 8; i++) keep[i] = st[i];
                    sha256_iv(st);
                    phase = 5;
                    b = 0;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 32; i++)
                    if (32 * (int)b + i < dgst_bytes) dg[32 * b + i] = (uint8_t)(st[i >> 2] >> (24 - 8 * (i & 3)));
                sha256_iv(st);
                if (++b == nm) break;
            }
        }
    }

    // H_msg = MGF1-SHA256(SHA256(R || PK || m), dgst) (hash_sha256.cu:200-262);
    // writes dgst_bytes bytes to dg (a byte array in registers/local).
    SPX_DEV static void mgf1_digest(uint8_t *dg, int dgst_bytes, const uint32_t seed[8]) {
        for (int c = 0; 32 * c < dgst_bytes; c++) {
            uint32_t w[16], s[8];
#pragma unroll
            for (int i = 0; i < 8; i++) w[i] = seed[i];
            w[8] = (uint32_t)c;
            w[9] = 0x80000000u;
#pragma unroll
            for (int i = 10; i < 15; i++) w[i] = 0;
            w[15] = 36 * 8;
            sha256_iv(s);
            sha256_compress(s, w);
            for (int i = 0; i < 32 && 32 * c + i < dgst_bytes; i++)
                dg[32 * c + i] = (uint8_t)(s[i >> 2] >> (24 - 8 * (i & 3)));
        }
    }
    SPX_DEV static void h_msg(uint8_t *dg, int dgst_bytes, const uint32_t R[W], const uint32_t pk[2 * W],
                              const uint8_t *m, uint64_t mlen) {
        uint32_t pre[3 * W];
#pragma unroll
        for (int i = 0; i < W; i++) pre[i] = R[i];
#pragma unroll
        for (int i = 0; i < 2 * W; i++) pre[W + i] = pk[i];
        uint32_t seed[8];
        sha256_iv(seed);
        stream_msg<3 * W>(seed, 0, pre, m, mlen);
        mgf1_digest(dg, dgst_bytes, seed);
    }
};

// ===========================================================================
// SHAKE-256 family (rate 136 bytes = 17 lanes, domain padding 0x1F..0x80)
// ===========================================================================
template <int N, bool ROBUST>
struct Shake {
    static constexpr int W = N / 4;
    static constexpr int NL = N / 8;  // lanes per value
    static constexpr bool kRobust = ROBUST;
    static constexpr int kShake = 1;
    static constexpr int kLeafMinBlocks = 1;

    SPX_DEV static void load(uint32_t v[W], const uint8_t *p) { load_bytes_le<N>(v, p); }
    SPX_DEV static void store(uint8_t *p, const uint32_t v[W]) { store_bytes_le<N>(p, v); }

    SPX_DEV static void key_init(KeyRegs<N> &k, const uint8_t *skseed, const uint8_t *pub) {
        load(k.skseed, skseed);
        load(k.pub, pub);
#pragma unroll
        for (int i = 0; i < 8; i++) k.mid[i] = 0;
    }

    SPX_DEV static uint64_t vlane(const uint32_t v[], int i) { return lane_of(v[2 * i], v[2 * i + 1]); }

    // SHAKE256(prefix(NL lanes) || ADRS(4 lanes) || in(L lanes)) -> NO lanes,
    // single permutation (every short input here is < 136 bytes)
    template <int L, int NO>
    SPX_DEV static void short_hash(uint64_t out[NO], const uint32_t pre[W], const Adrs &a, const uint64_t *in) {
        static_assert(8 * (NL + 4 + L) < 136, "short input must fit one block");
        uint64_t A[25];
        uint64_t al[4];
        adrs_lanes(a, al);
#pragma unroll
        for (int i = 0; i < 25; i++) A[i] = 0;
#pragma unroll
        for (int i = 0; i < NL; i++) A[i] = vlane(pre, i);
#pragma unroll
        for (int i = 0; i < 4; i++) A[NL + i] = al[i];
#pragma unroll
        for (int i = 0; i < L; i++) A[NL + 4 + i] = in[i];
        A[NL + 4 + L] = 0x1Full;
        A[16] ^= 0x8000000000000000ull;
        keccak_f1600(A);
#pragma unroll
        for (int i = 0; i < NO; i++) out[i] = A[i];
    }

    template <int L>
    SPX_DEV static void thash(uint32_t out[W], const KeyRegs<N> &k, const Adrs &a, const uint32_t in[2 * L]) {
        uint64_t x[L];
#pragma unroll
        for (int i = 0; i < L; i++) x[i] = vlane(in, i);
        if (ROBUST) {
            uint64_t mk[L];
            short_hash<0, L>(mk, k.pub, a, x);
#pragma unroll
            for (int i = 0; i < L; i++) x[i] ^= mk[i];
        }
        uint64_t o[NL];
        short_hash<L, NL>(o, k.pub, a, x);
#pragma unroll
        for (int i = 0; i < NL; i++) { out[2 * i] = (uint32_t)o[i]; out[2 * i + 1] = (uint32_t)(o[i] >> 32); }
    }

    SPX_DEV static void F(uint32_t out[W], const uint32_t in[W], const Adrs &a, const KeyRegs<N> &k) {
        thash<NL>(out, k, a, in);
    }
    SPX_DEV static void H(uint32_t out[W], const uint32_t l[W], const uint32_t r[W], const Adrs &a,
                          const KeyRegs<N> &k) {
        uint32_t t[2 * W];
#pragma unroll
        for (int i = 0; i < W; i++) { t[i] = l[i]; t[W + i] = r[i]; }
        thash<2 * NL>(out, k, a, t);
    }
    // WOTS+ chain steps: a Keccak permutation has no reusable prefix, so the
    // prepared chain is just its address
    struct FCtx {
        Adrs a;
    };
    SPX_DEV static void f_prepare(FCtx &f, const Adrs &a, const KeyRegs<N> &) { f.a = a; }
    SPX_DEV static void f_step(uint32_t out[W], const uint32_t in[W], const FCtx &f, uint32_t hash,
                               const KeyRegs<N> &k) {
        Adrs a = f.a;
        adrs_hash(a, hash);
        F(out, in, a, k);
    }

    // PRF = SHAKE256(SK_SEED || ADRS) (hash_shake256.cu:38-47)
    SPX_DEV static void PRF(uint32_t out[W], const Adrs &a, const KeyRegs<N> &k) {
        uint64_t o[NL];
        uint64_t dummy[1] = {0};
        short_hash<0, NL>(o, k.skseed, a, dummy);
#pragma unroll
        for (int i = 0; i < NL; i++) { out[2 * i] = (uint32_t)o[i]; out[2 * i + 1] = (uint32_t)(o[i] >> 32); }
    }

    // T_l streaming: PUB_SEED || ADRS || v_0 || v_1 ...  (lanes, rate 17)
    // buf: per-thread shared memory, kSmemWords words (17 lanes + robust mask block)
    static constexpr int kSmemWords = 2 * 17 + (ROBUST ? 2 * 17 : 0);
    struct TStream {
        uint64_t A[25];
        uint64_t *buf;   // 17 lanes
        int pos;         // lanes filled in buf
        // robust: mask sponge squeezed 17 lanes at a time
        uint64_t M[25];
        int mpos;
    };
    SPX_DEV static void t_init(TStream &t, uint32_t *smem, const KeyRegs<N> &k, const Adrs &a) {
        t.buf = reinterpret_cast<uint64_t *>(smem);
#pragma unroll
        for (int i = 0; i < 25; i++) t.A[i] = 0;
        uint64_t al[4];
        adrs_lanes(a, al);
#pragma unroll
        for (int i = 0; i < NL; i++) t.buf[i] = vlane(k.pub, i);
#pragma unroll
        for (int i = 0; i < 4; i++) t.buf[NL + i] = al[i];
        t.pos = NL + 4;
        if (ROBUST) {
            // mask = SHAKE256(PUB_SEED || ADRS, .): absorb + first permutation
#pragma unroll
            for (int i = 0; i < 25; i++) t.M[i] = 0;
#pragma unroll
            for (int i = 0; i < NL; i++) t.M[i] = vlane(k.pub, i);
#pragma unroll
            for (int i = 0; i < 4; i++) t.M[NL + i] = al[i];
            t.M[NL + 4] = 0x1Full;
            t.M[16] ^= 0x8000000000000000ull;
            keccak_f1600(t.M);
            uint64_t *mb = t.buf + 17;
#pragma unroll
            for (int i = 0; i < 17; i++) mb[i] = t.M[i];
            t.mpos = 0;
        }
    }
    SPX_DEV static void t_flush(TStream &t) {
#pragma unroll
        for (int i = 0; i < 17; i++) t.A[i] ^= t.buf[i];
        keccak_f1600(t.A);
    }
    SPX_DEV static void t_lane(TStream &t, uint64_t x) {
        if (ROBUST) {
            uint64_t *mb = t.buf + 17;
            if (t.mpos == 17) {
                keccak_f1600(t.M);
#pragma unroll
                for (int i = 0; i < 17; i++) mb[i] = t.M[i];
                t.mpos = 0;
            }
            x ^= mb[t.mpos++];
        }
        t.buf[t.pos++] = x;
        if (t.pos == 17) {
            t_flush(t);
            t.pos = 0;
        }
    }
    SPX_DEV static void t_absorb(TStream &t, const uint32_t v[W], const KeyRegs<N> &) {
#pragma unroll
        for (int i = 0; i < NL; i++) t_lane(t, vlane(v, i));
    }
    SPX_DEV static void t_final(uint32_t out[W], TStream &t) {
        for (int i = t.pos; i < 17; i++) t.buf[i] = 0;
        t.buf[t.pos] ^= 0x1Full;
        t.buf[16] ^= 0x8000000000000000ull;
        t_flush(t);
#pragma unroll
        for (int i = 0; i < NL; i++) { out[2 * i] = (uint32_t)t.A[i]; out[2 * i + 1] = (uint32_t)(t.A[i] >> 32); }
    }

    // ---- message hashing --------------------------------------------------
    // lane q (little-endian) of m with the SHAKE padding byte 0x1F at mlen;
    // m must be 8-byte aligned and readable up to the next multiple of 8.
    SPX_DEV static uint64_t msg_lane(const uint8_t *m, uint64_t mlen, uint64_t q) {
        uint64_t b = 8 * q;
        if (b + 8 <= mlen) return *reinterpret_cast<const uint64_t *>(m + b);
        if (b > mlen) return 0;
        uint32_t keep = (uint32_t)(mlen - b);  // 0..7
        uint64_t x = keep ? *reinterpret_cast<const uint64_t *>(m + b) : 0ull;
        uint64_t lo = keep ? (0xffffffffffffffffull >> (64 - 8 * keep)) : 0ull;
        return (x & lo) | (0x1Full << (8 * keep));
    }
    // SHAKE256(prefix(P lanes) || m) absorbed into A (state after the last
    // permutation).  Blocks wholly inside the message are loaded one block
    // ahead of the permutation (m + 8 * lane is 8-byte aligned).
    template <int P>
    SPX_DEV static void stream_msg(uint64_t A[25], const uint64_t pre[P], const uint8_t *m, uint64_t mlen) {
        const uint64_t dbytes = 8 * (uint64_t)P + mlen;
        const uint64_t nblocks = dbytes / 136 + 1;
        constexpr int PB = (P + 16) / 17;
        auto full = [&](uint64_t b) { return b >= (uint64_t)PB && 8 * (17 * b - P + 17) <= mlen; };
        uint64_t nxt[17];
        bool have = false;
#pragma unroll
        for (int i = 0; i < 25; i++) A[i] = 0;
        for (uint64_t b = 0; b < nblocks; b++) {
            if (have) {
#pragma unroll
                for (int j = 0; j < 17; j++) A[j] ^= nxt[j];
            } else if (b < PB) {
#pragma unroll
                for (int pb = 0; pb < PB; pb++) {
                    if (pb == (int)b) {
#pragma unroll
                        for (int j = 0; j < 17; j++) {
                            const int g = 17 * pb + j;
                            A[j] ^= g < P ? pre[g < P ? g : 0] : msg_lane(m, mlen, (uint64_t)(g - P));
                        }
                    }
                }
            } else {
                const uint64_t q0 = 17 * b - P;
#pragma unroll
                for (int j = 0; j < 17; j++) A[j] ^= msg_lane(m, mlen, q0 + j);
            }
            have = b + 1 < nblocks && full(b + 1);
            if (have) {
                const uint64_t *p = reinterpret_cast<const uint64_t *>(m + 8 * (17 * (b + 1) - P));
#pragma unroll
                for (int j = 0; j < 17; j++) nxt[j] = p[j];
            }
            // the 0x1F byte comes from msg_lane (the lane holding byte mlen is
            // always inside the last block); the final 0x80 is added here
            if (b == nblocks - 1) A[16] ^= 0x8000000000000000ull;
            keccak_f1600(A);
        }
    }

    // PRF_msg = SHAKE256(SK_PRF || optrand || m, n) (hash_shake256.cu:64-77)
    SPX_DEV static void prf_msg(uint32_t R[W], const uint32_t skprf[W], const uint32_t optrand[W],
                                const uint8_t *m, uint64_t mlen) {
        uint64_t pre[2 * NL], A[25];
#pragma unroll
        for (int i = 0; i < NL; i++) { pre[i] = vlane(skprf, i); pre[NL + i] = vlane(optrand, i); }
        stream_msg<2 * NL>(A, pre, m, mlen);
#pragma unroll
        for (int i = 0; i < NL; i++) { R[2 * i] = (uint32_t)A[i]; R[2 * i + 1] = (uint32_t)(A[i] >> 32); }
    }
    // H_msg = SHAKE256(R || PK || m, dgst) (hash_shake256.cu:96-130)
    SPX_DEV static void h_msg(uint8_t *dg, int dgst_bytes, const uint32_t R[W], const uint32_t pk[2 * W],
                              const uint8_t *m, uint64_t mlen) {
        uint64_t pre[3 * NL], A[25];
#pragma unroll
        for (int i = 0; i < NL; i++) pre[i] = vlane(R, i);
#pragma unroll
        for (int i = 0; i < 2 * NL; i++) pre[NL + i] = vlane(pk, i);
        stream_msg<3 * NL>(A, pre, m, mlen);
        for (int i = 0; i < dgst_bytes; i++) dg[i] = (uint8_t)(A[i >> 3] >> (8 * (i & 7)));
    }
};

}  // namespace cuspx
