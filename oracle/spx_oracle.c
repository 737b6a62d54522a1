/*
 * spx_oracle.c -- CPU restatement of the reference SPHINCS+ path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine and the CPU
 * baseline.  The product library never links this file.
 *
 * Each function names the reference function it restates (file:line in the
 * reference tree).  Arithmetic follows the reference exactly, including its
 * departures from FIPS 205: SHA-256 at every security level, a 22-byte
 * compressed ADRS for SHA-256 and the same SHA-256 byte offsets inside a
 * 32-byte ADRS for SHAKE-256 (params.h:148, sha256_offsets.h:9-17),
 * H_msg = MGF1-SHA256(SHA256(R||PK||M)), LSB-first FORS indices.
 * The robust tweakable hash (absent from the reference) follows the
 * published SPHINCS+ round-3 robust construction; its parity is unpinned.
 */
#include "spx_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------ */
/* parameters (params.h:33-146)                                             */
/* ------------------------------------------------------------------------ */

int spxo_params_init(spxo_params *p, int hash, int robust, int n, int h, int d, int a, int k)
{
    if (hash != SPXO_SHA256 && hash != SPXO_SHAKE256) return -1;
    if (n != 16 && n != 24 && n != 32) return -1;
    if (d <= 0 || h % d != 0 || a <= 0 || a > 16 || k <= 0 || k > 64) return -1;
    memset(p, 0, sizeof(*p));
    p->hash = hash; p->robust = robust ? 1 : 0;
    p->n = n; p->h = h; p->d = d; p->a = a; p->k = k; p->w = 16;
    p->hp = h / d;
    if (p->hp > 16 || p->hp * (d - 1) > 64) return -1;
    p->len1 = 2 * n;               /* 8n / log2(w), params.h:101 */
    p->len2 = 3;                   /* w=16, 8 < n <= 136, params.h:116-117 */
    p->len = p->len1 + p->len2;
    p->fors_msg_bytes = (a * k + 7) / 8;
    p->fors_bytes = (a + 1) * k * n;
    p->wots_bytes = p->len * n;
    p->sig_bytes = n + p->fors_bytes + d * p->wots_bytes + h * n;  /* params.h:138 */
    p->pk_bytes = 2 * n;
    p->sk_bytes = 4 * n;
    p->seed_bytes = 3 * n;
    p->tree_bits = p->hp * (d - 1);                     /* hash_sha256.cu:204 */
    p->tree_bytes = (p->tree_bits + 7) / 8;
    p->leaf_bits = p->hp;
    p->leaf_bytes = (p->leaf_bits + 7) / 8;
    p->dgst_bytes = p->fors_msg_bytes + p->tree_bytes + p->leaf_bytes;
    return 0;
}

int spxo_params_from_name(spxo_params *p, const char *name)
{
    static const struct { const char *tag; int n, h, d, a, k; } T[] = {
        {"128s", 16, 63, 7, 12, 14}, {"128f", 16, 66, 22, 6, 33},
        {"192s", 24, 63, 7, 14, 17}, {"192f", 24, 66, 22, 8, 33},
        {"256s", 32, 64, 8, 14, 22}, {"256f", 32, 68, 17, 9, 35},
    };
    int hash, robust;
    const char *rest;
    if (!strncmp(name, "sha256-", 7)) { hash = SPXO_SHA256; rest = name + 7; }
    else if (!strncmp(name, "shake256-", 9)) { hash = SPXO_SHAKE256; rest = name + 9; }
    else return -1;
    if (strlen(rest) < 4) return -1;
    const char *mode = rest + 4;
    if (!strcmp(mode, "") || !strcmp(mode, "-simple")) robust = 0;
    else if (!strcmp(mode, "-robust")) robust = 1;
    else return -1;
    for (size_t i = 0; i < sizeof(T) / sizeof(T[0]); i++)
        if (!strncmp(rest, T[i].tag, 4))
            return spxo_params_init(p, hash, robust, T[i].n, T[i].h, T[i].d, T[i].a, T[i].k);
    return -1;
}

/* ------------------------------------------------------------------------ */
/* SHA-256 (FIPS 180-4), restating sha256.cu:103-405                        */
/* ------------------------------------------------------------------------ */

static const uint32_t K256[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2,
};
static const uint32_t IV256[8] = {
    0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a, 0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19,
};

static inline uint32_t rotr32(uint32_t x, int c) { return (x >> c) | (x << (32 - c)); }
static inline uint32_t be32(const uint8_t *p)
{
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
static inline void put_be32(uint8_t *p, uint32_t v)
{
    p[0] = (uint8_t)(v >> 24); p[1] = (uint8_t)(v >> 16); p[2] = (uint8_t)(v >> 8); p[3] = (uint8_t)v;
}

/* Hash-unit counters of the calling thread: [0] SHA-256 compressions,
 * [1] Keccak-f[1600] permutations, [2] the units of both spent inside
 * wots_sign (the reference recomputes the signing leaf's chains there).
 * Test infrastructure: they pin the work model behind the benchmark's
 * roofline fractions. */
static _Thread_local unsigned long long g_units[3];
void spxo_units(unsigned long long out[3]) { memcpy(out, g_units, sizeof g_units); }
void spxo_units_reset(void) { memset(g_units, 0, sizeof g_units); }

/* one 64-byte block (crypto_hashblocks_sha256, sha256.cu:103-259) */
static void sha256_block(uint32_t s[8], const uint8_t *blk)
{
    uint32_t w[64];
    g_units[0]++;
    for (int i = 0; i < 16; i++) w[i] = be32(blk + 4 * i);
    for (int i = 16; i < 64; i++) {
        uint32_t s0 = rotr32(w[i - 15], 7) ^ rotr32(w[i - 15], 18) ^ (w[i - 15] >> 3);
        uint32_t s1 = rotr32(w[i - 2], 17) ^ rotr32(w[i - 2], 19) ^ (w[i - 2] >> 10);
        w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = s[0], b = s[1], c = s[2], d = s[3], e = s[4], f = s[5], g = s[6], h = s[7];
    for (int i = 0; i < 64; i++) {
        uint32_t t1 = h + (rotr32(e, 6) ^ rotr32(e, 11) ^ rotr32(e, 25)) + ((e & f) ^ (~e & g)) + K256[i] + w[i];
        uint32_t t2 = (rotr32(a, 2) ^ rotr32(a, 13) ^ rotr32(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
        h = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    s[0] += a; s[1] += b; s[2] += c; s[3] += d; s[4] += e; s[5] += f; s[6] += g; s[7] += h;
}

/* incremental state: chaining value + bytes absorbed so far (the reference's
 * 40-byte state, sha256.cu:268-287) */
typedef struct { uint32_t h[8]; uint64_t bytes; } sha256_ctx;

static void sha256_init(sha256_ctx *c)
{
    memcpy(c->h, IV256, sizeof(IV256));
    c->bytes = 0;
}

/* absorb whole blocks (sha256_inc_blocks, sha256.cu:278-287) */
static void sha256_blocks(sha256_ctx *c, const uint8_t *in, size_t nblocks)
{
    for (size_t i = 0; i < nblocks; i++) sha256_block(c->h, in + 64 * i);
    c->bytes += 64 * (uint64_t)nblocks;
}

/* absorb the tail and pad (sha256_inc_finalize, sha256.cu:289-347) */
static void sha256_final(sha256_ctx *c, uint8_t out[32], const uint8_t *in, size_t inlen)
{
    uint8_t pad[128];
    uint64_t bits = (c->bytes + inlen) * 8;
    size_t full = inlen / 64;
    sha256_blocks(c, in, full);
    in += 64 * full; inlen -= 64 * full;
    memset(pad, 0, sizeof(pad));
    memcpy(pad, in, inlen);
    pad[inlen] = 0x80;
    size_t total = inlen < 56 ? 64 : 128;
    for (int i = 0; i < 8; i++) pad[total - 1 - i] = (uint8_t)(bits >> (8 * i));
    for (size_t off = 0; off < total; off += 64) sha256_block(c->h, pad + off);
    for (int i = 0; i < 8; i++) put_be32(out + 4 * i, c->h[i]);
}

void spxo_sha256(uint8_t out[32], const uint8_t *in, size_t inlen)
{
    sha256_ctx c;
    sha256_init(&c);
    sha256_final(&c, out, in, inlen);
}

/* MGF1-SHA256 (sha256.cu:362-383): out = SHA256(in||BE32(0)) || SHA256(in||BE32(1)) ... */
void spxo_mgf1(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen)
{
    uint8_t stackbuf[128];
    uint8_t *buf = inlen + 4 <= sizeof(stackbuf) ? stackbuf : (uint8_t *)malloc(inlen + 4);
    uint8_t blk[32];
    memcpy(buf, in, inlen);
    for (uint32_t i = 0; outlen > 0; i++) {
        put_be32(buf + inlen, i);
        spxo_sha256(blk, buf, inlen + 4);
        size_t take = outlen < 32 ? outlen : 32;
        memcpy(out, blk, take);
        out += take; outlen -= take;
    }
    if (buf != stackbuf) free(buf);
}

/* ------------------------------------------------------------------------ */
/* Keccak-f[1600] and SHAKE-256 (FIPS 202), restating fips202.cu:71-660     */
/* ------------------------------------------------------------------------ */

static uint64_t KRC[24];
static int KROT[25];
static int keccak_ready;

/* round constants from the FIPS 202 rc(t) LFSR, rotation offsets from the
 * (x,y) -> (y, 2x+3y) walk; computed once instead of tabulated */
static void keccak_tables(void)
{
    if (keccak_ready) return;
    uint8_t lfsr = 1;
    for (int r = 0; r < 24; r++) {
        uint64_t rc = 0;
        for (int j = 0; j < 7; j++) {
            if (lfsr & 1) rc |= 1ULL << ((1 << j) - 1);
            lfsr = (uint8_t)((lfsr << 1) ^ ((lfsr & 0x80) ? 0x71 : 0));
        }
        KRC[r] = rc;
    }
    int x = 1, y = 0;
    KROT[0] = 0;
    for (int t = 0; t < 24; t++) {
        KROT[x + 5 * y] = ((t + 1) * (t + 2) / 2) % 64;
        int nx = y, ny = (2 * x + 3 * y) % 5;
        x = nx; y = ny;
    }
    keccak_ready = 1;
}

static inline uint64_t rotl64(uint64_t v, int c) { return c ? (v << c) | (v >> (64 - c)) : v; }

static void keccak_f1600(uint64_t s[25])
{
    g_units[1]++;
    for (int r = 0; r < 24; r++) {
        uint64_t C[5], D[5], B[25];
        for (int x = 0; x < 5; x++) C[x] = s[x] ^ s[x + 5] ^ s[x + 10] ^ s[x + 15] ^ s[x + 20];
        for (int x = 0; x < 5; x++) D[x] = C[(x + 4) % 5] ^ rotl64(C[(x + 1) % 5], 1);
        for (int i = 0; i < 25; i++) s[i] ^= D[i % 5];
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++)
                B[y + 5 * ((2 * x + 3 * y) % 5)] = rotl64(s[x + 5 * y], KROT[x + 5 * y]);
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++)
                s[x + 5 * y] = B[x + 5 * y] ^ (~B[(x + 1) % 5 + 5 * y] & B[(x + 2) % 5 + 5 * y]);
        s[0] ^= KRC[r];
    }
}

#define SHAKE256_RATE 136
typedef struct { uint64_t s[25]; size_t pos; } shake_ctx;

static void shake_init(shake_ctx *c) { keccak_tables(); memset(c, 0, sizeof(*c)); }
static void shake_absorb(shake_ctx *c, const uint8_t *in, size_t len)
{
    while (len--) {
        c->s[c->pos / 8] ^= (uint64_t)(*in++) << (8 * (c->pos % 8));
        if (++c->pos == SHAKE256_RATE) { keccak_f1600(c->s); c->pos = 0; }
    }
}
static void shake_finalize(shake_ctx *c)
{
    c->s[c->pos / 8] ^= (uint64_t)0x1F << (8 * (c->pos % 8));
    c->s[(SHAKE256_RATE - 1) / 8] ^= (uint64_t)0x80 << (8 * ((SHAKE256_RATE - 1) % 8));
    keccak_f1600(c->s);
    c->pos = 0;
}
static void shake_squeeze(shake_ctx *c, uint8_t *out, size_t len)
{
    while (len--) {
        if (c->pos == SHAKE256_RATE) { keccak_f1600(c->s); c->pos = 0; }
        *out++ = (uint8_t)(c->s[c->pos / 8] >> (8 * (c->pos % 8)));
        c->pos++;
    }
}

void spxo_shake256(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen)
{
    shake_ctx c;
    shake_init(&c);
    shake_absorb(&c, in, inlen);
    shake_finalize(&c);
    shake_squeeze(&c, out, outlen);
}

/* ------------------------------------------------------------------------ */
/* ADRS byte layout (address.cu:10-180 with sha256_offsets.h:9-17)          */
/* ------------------------------------------------------------------------ */

enum { OFF_LAYER = 0, OFF_TREE = 1, OFF_TYPE = 9, OFF_KP2 = 12, OFF_KP1 = 13,
       OFF_CHAIN = 17, OFF_HASH = 21, OFF_HGT = 17, OFF_IDX = 18 };
enum { T_WOTS = 0, T_WOTSPK = 1, T_HASHTREE = 2, T_FORSTREE = 3, T_FORSPK = 4 };

static void set_layer(uint8_t a[32], uint32_t v) { a[OFF_LAYER] = (uint8_t)v; }
static void set_tree(uint8_t a[32], uint64_t t)
{
    for (int i = 7; i >= 0; i--) { a[OFF_TREE + i] = (uint8_t)t; t >>= 8; }
}
static void set_type(uint8_t a[32], uint32_t v) { a[OFF_TYPE] = (uint8_t)v; }
/* set_keypair_addr (address.cu:80-88): the high byte is written only when a
 * subtree has more than 256 leaves; below that it is always zero anyway */
static void set_keypair(const spxo_params *p, uint8_t a[32], uint32_t kp)
{
    if (p->hp > 8) a[OFF_KP2] = (uint8_t)(kp >> 8);
    a[OFF_KP1] = (uint8_t)kp;
}
static void set_chain(uint8_t a[32], uint32_t v) { a[OFF_CHAIN] = (uint8_t)v; }
static void set_hash(uint8_t a[32], uint32_t v) { a[OFF_HASH] = (uint8_t)v; }
static void set_height(uint8_t a[32], uint32_t v) { a[OFF_HGT] = (uint8_t)v; }
static void set_index(uint8_t a[32], uint32_t v) { put_be32(a + OFF_IDX, v); }
/* copy_subtree_addr: layer + tree bytes 0..8 */
static void copy_subtree(uint8_t o[32], const uint8_t i[32]) { memcpy(o, i, OFF_TREE + 8); }
/* copy_keypair_addr: layer + tree + keypair bytes */
static void copy_keypair(const spxo_params *p, uint8_t o[32], const uint8_t i[32])
{
    memcpy(o, i, OFF_TREE + 8);
    if (p->hp > 8) o[OFF_KP2] = i[OFF_KP2];
    o[OFF_KP1] = i[OFF_KP1];
}

/* ------------------------------------------------------------------------ */
/* tweakable hash, PRF, PRF_msg, H_msg                                      */
/* ------------------------------------------------------------------------ */

#define SHA256_ADDR_BYTES 22

/* hashing context: the reference's initialize_hash_function/seed_state
 * (hash_sha256.cu:19-31, sha256.cu:391-405) made explicit and per key */
typedef struct {
    const spxo_params *p;
    const uint8_t *pub_seed;
    const uint8_t *sk_seed;
    sha256_ctx seeded;   /* SHA-256 state after PUB_SEED || 0^(64-n) */
} hctx;

static void hctx_init(hctx *h, const spxo_params *p, const uint8_t *pub_seed, const uint8_t *sk_seed)
{
    h->p = p; h->pub_seed = pub_seed; h->sk_seed = sk_seed;
    if (p->hash == SPXO_SHA256) {
        uint8_t blk[64];
        memset(blk, 0, 64);
        memcpy(blk, pub_seed, p->n);
        sha256_init(&h->seeded);
        sha256_blocks(&h->seeded, blk, 1);
    }
}

/* thash (thash_sha256.cu:16-34 / thash_shake256.cu:15-25 simple; robust
 * restated from the SPHINCS+ round-3 robust construction) */
/* largest tweakable-hash input: T_len with len=67 chains of n=32 bytes */
#define THASH_MAX_IN (80 * 32)

static void thash_ctx(const hctx *hc, uint8_t *out, const uint8_t *in, unsigned inblocks, const uint8_t addr[32])
{
    const spxo_params *p = hc->p;
    const int n = p->n;
    const size_t inlen = (size_t)inblocks * n;
    uint8_t buf[32 + 32 + THASH_MAX_IN + 4];
    uint8_t mask[THASH_MAX_IN];
    if (p->hash == SPXO_SHA256) {
        uint8_t outbuf[32];
        memcpy(buf, hc->pub_seed, n);
        memcpy(buf + n, addr, SHA256_ADDR_BYTES);
        if (p->robust) {
            /* bitmask = MGF1-SHA256(PUB_SEED || ADRS_c, inblocks*n) */
            spxo_mgf1(mask, inlen, buf, n + SHA256_ADDR_BYTES);
            for (size_t i = 0; i < inlen; i++) buf[n + SHA256_ADDR_BYTES + i] = in[i] ^ mask[i];
        } else {
            memcpy(buf + n + SHA256_ADDR_BYTES, in, inlen);
        }
        sha256_ctx c = hc->seeded;
        sha256_final(&c, outbuf, buf + n, SHA256_ADDR_BYTES + inlen);
        memcpy(out, outbuf, n);
    } else {
        memcpy(buf, hc->pub_seed, n);
        memcpy(buf + n, addr, 32);
        if (p->robust) {
            /* bitmask = SHAKE256(PUB_SEED || ADRS, inblocks*n) */
            spxo_shake256(mask, inlen, buf, n + 32);
            for (size_t i = 0; i < inlen; i++) buf[n + 32 + i] = in[i] ^ mask[i];
        } else {
            memcpy(buf + n + 32, in, inlen);
        }
        spxo_shake256(out, n, buf, n + 32 + inlen);
    }
}

void spxo_thash(const spxo_params *p, uint8_t *out, const uint8_t *in, unsigned inblocks,
                const uint8_t *pub_seed, const uint8_t addr[32])
{
    hctx h;
    hctx_init(&h, p, pub_seed, NULL);
    thash_ctx(&h, out, in, inblocks, addr);
}

/* prf_addr (hash_sha256.cu:65-89, hash_shake256.cu:38-58) */
static void prf_addr(const hctx *hc, uint8_t *out, const uint8_t addr[32])
{
    const spxo_params *p = hc->p;
    uint8_t buf[32 + 32], outbuf[32];
    memcpy(buf, hc->sk_seed, p->n);
    if (p->hash == SPXO_SHA256) {
        memcpy(buf + p->n, addr, SHA256_ADDR_BYTES);
        spxo_sha256(outbuf, buf, p->n + SHA256_ADDR_BYTES);
        memcpy(out, outbuf, p->n);
    } else {
        memcpy(buf + p->n, addr, 32);
        spxo_shake256(out, p->n, buf, p->n + 32);
    }
}

/* gen_message_random: HMAC-SHA256(SK.prf, optrand||m) (hash_sha256.cu:99-145)
 * or SHAKE256(SK.prf||optrand||m) (hash_shake256.cu:64-77) */
void spxo_gen_message_random(const spxo_params *p, uint8_t *R, const uint8_t *sk_prf,
                             const uint8_t *optrand, const uint8_t *m, size_t mlen)
{
    const int n = p->n;
    if (p->hash == SPXO_SHA256) {
        uint8_t blk[64], inner[32], outer[64 + 32], res[32];
        sha256_ctx c;
        for (int i = 0; i < 64; i++) blk[i] = (uint8_t)((i < n ? sk_prf[i] : 0) ^ 0x36);
        sha256_init(&c);
        sha256_blocks(&c, blk, 1);
        /* absorb optrand || m */
        uint8_t *buf = (uint8_t *)malloc(n + mlen + 1);
        memcpy(buf, optrand, n);
        if (mlen) memcpy(buf + n, m, mlen);
        sha256_final(&c, inner, buf, n + mlen);
        free(buf);
        for (int i = 0; i < 64; i++) outer[i] = (uint8_t)((i < n ? sk_prf[i] : 0) ^ 0x5c);
        memcpy(outer + 64, inner, 32);
        spxo_sha256(res, outer, 96);
        memcpy(R, res, n);
    } else {
        shake_ctx c;
        shake_init(&c);
        shake_absorb(&c, sk_prf, n);
        shake_absorb(&c, optrand, n);
        shake_absorb(&c, m, mlen);
        shake_finalize(&c);
        shake_squeeze(&c, R, n);
    }
}

static uint64_t be_bytes(const uint8_t *in, int len)
{
    uint64_t v = 0;
    for (int i = 0; i < len; i++) v = (v << 8) | in[i];
    return v;
}

/* hash_message (hash_sha256.cu:200-262, hash_shake256.cu:96-130) */
void spxo_hash_message(const spxo_params *p, uint8_t *digest, uint64_t *tree, uint32_t *leaf_idx,
                       const uint8_t *R, const uint8_t *pk, const uint8_t *m, size_t mlen)
{
    const int n = p->n;
    uint8_t buf[128];
    if (p->hash == SPXO_SHA256) {
        uint8_t seed[32];
        sha256_ctx c;
        uint8_t *tmp = (uint8_t *)malloc(3 * n + mlen + 1);
        memcpy(tmp, R, n);
        memcpy(tmp + n, pk, 2 * n);
        if (mlen) memcpy(tmp + 3 * n, m, mlen);
        sha256_init(&c);
        sha256_final(&c, seed, tmp, 3 * n + mlen);
        free(tmp);
        spxo_mgf1(buf, p->dgst_bytes, seed, 32);
    } else {
        shake_ctx c;
        shake_init(&c);
        shake_absorb(&c, R, n);
        shake_absorb(&c, pk, 2 * n);
        shake_absorb(&c, m, mlen);
        shake_finalize(&c);
        shake_squeeze(&c, buf, p->dgst_bytes);
    }
    memcpy(digest, buf, p->fors_msg_bytes);
    uint64_t t = be_bytes(buf + p->fors_msg_bytes, p->tree_bytes);
    *tree = p->tree_bits == 64 ? t : (t & ((~(uint64_t)0) >> (64 - p->tree_bits)));
    uint32_t l = (uint32_t)be_bytes(buf + p->fors_msg_bytes + p->tree_bytes, p->leaf_bytes);
    *leaf_idx = l & ((~(uint32_t)0) >> (32 - p->leaf_bits));
}

/* ------------------------------------------------------------------------ */
/* WOTS+ (wots.cu:24-197, 614-641, 777-804)                                 */
/* ------------------------------------------------------------------------ */

/* gen_chain (wots.cu:51-62) */
static void gen_chain(const hctx *hc, uint8_t *out, const uint8_t *in, unsigned start, unsigned steps, uint8_t addr[32])
{
    memcpy(out, in, hc->p->n);
    for (unsigned i = start; i < start + steps && i < 16; i++) {
        set_hash(addr, i);
        thash_ctx(hc, out, out, 1, addr);
    }
}

/* chain_lengths = base_w(msg) || base_w(checksum) (wots.cu:84-166): digits
 * MSB-nibble first, checksum left-shifted so its unused bits are the LSBs */
static void chain_lengths(const spxo_params *p, unsigned *len, const uint8_t *msg)
{
    unsigned csum = 0;
    for (int i = 0; i < p->len1; i++) {
        len[i] = (i & 1) ? (msg[i / 2] & 15) : (msg[i / 2] >> 4);
        csum += 15 - len[i];
    }
    int shift = (8 - ((p->len2 * 4) % 8)) % 8;
    csum <<= shift;
    int cbytes = (p->len2 * 4 + 7) / 8;
    uint8_t cb[8];
    for (int i = cbytes - 1; i >= 0; i--) { cb[i] = (uint8_t)csum; csum >>= 8; }
    for (int i = 0; i < p->len2; i++)
        len[p->len1 + i] = (i & 1) ? (cb[i / 2] & 15) : (cb[i / 2] >> 4);
}

/* wots_gen_pk (wots.cu:176-185) with wots_gen_sk (wots.cu:24-31) */
static void wots_gen_pk(const hctx *hc, uint8_t *pk, uint8_t addr[32])
{
    const int n = hc->p->n;
    for (int i = 0; i < hc->p->len; i++) {
        set_chain(addr, i);
        set_hash(addr, 0);
        prf_addr(hc, pk + i * n, addr);
        gen_chain(hc, pk + i * n, pk + i * n, 0, 15, addr);
    }
}

/* wots_sign (wots.cu:614-625) */
static void wots_sign(const hctx *hc, uint8_t *sig, const uint8_t *msg, uint8_t addr[32])
{
    const int n = hc->p->n;
    unsigned len[80];
    const unsigned long long before = g_units[0] + g_units[1];
    chain_lengths(hc->p, len, msg);
    for (int i = 0; i < hc->p->len; i++) {
        set_chain(addr, i);
        set_hash(addr, 0);
        prf_addr(hc, sig + i * n, addr);
        gen_chain(hc, sig + i * n, sig + i * n, 0, len[i], addr);
    }
    g_units[2] += g_units[0] + g_units[1] - before;
}

/* wots_pk_from_sig (wots.cu:777-789) */
static void wots_pk_from_sig(const hctx *hc, uint8_t *pk, const uint8_t *sig, const uint8_t *msg, uint8_t addr[32])
{
    const int n = hc->p->n;
    unsigned len[80];
    chain_lengths(hc->p, len, msg);
    for (int i = 0; i < hc->p->len; i++) {
        set_chain(addr, i);
        gen_chain(hc, pk + i * n, sig + i * n, len[i], 15 - len[i], addr);
    }
}

/* wots_gen_leaf (sign.cu:87-102) */
static void wots_gen_leaf(const hctx *hc, uint8_t *leaf, uint32_t addr_idx, const uint8_t tree_addr[32])
{
    const spxo_params *p = hc->p;
    uint8_t pk[80 * 32];
    uint8_t wa[32] = {0}, wpa[32] = {0};
    set_type(wa, T_WOTS);
    set_type(wpa, T_WOTSPK);
    copy_subtree(wa, tree_addr);
    set_keypair(p, wa, addr_idx);
    wots_gen_pk(hc, pk, wa);
    copy_keypair(p, wpa, wa);
    thash_ctx(hc, leaf, pk, p->len, wpa);
}

/* ------------------------------------------------------------------------ */
/* Merkle trees (utils.cu:94-241)                                           */
/* ------------------------------------------------------------------------ */

typedef void (*gen_leaf_fn)(const hctx *, uint8_t *, uint32_t, const uint8_t *);

/* compute_root (utils.cu:94-135) */
static void compute_root(const hctx *hc, uint8_t *root, const uint8_t *leaf, uint32_t leaf_idx,
                         uint32_t idx_offset, const uint8_t *auth, uint32_t height, uint8_t addr[32])
{
    const int n = hc->p->n;
    uint8_t buf[64];
    if (leaf_idx & 1) { memcpy(buf + n, leaf, n); memcpy(buf, auth, n); }
    else { memcpy(buf, leaf, n); memcpy(buf + n, auth, n); }
    auth += n;
    for (uint32_t i = 0; i < height - 1; i++) {
        leaf_idx >>= 1; idx_offset >>= 1;
        set_height(addr, i + 1);
        set_index(addr, leaf_idx + idx_offset);
        if (leaf_idx & 1) { thash_ctx(hc, buf + n, buf, 2, addr); memcpy(buf, auth, n); }
        else { thash_ctx(hc, buf, buf, 2, addr); memcpy(buf + n, auth, n); }
        auth += n;
    }
    leaf_idx >>= 1; idx_offset >>= 1;
    set_height(addr, height);
    set_index(addr, leaf_idx + idx_offset);
    thash_ctx(hc, root, buf, 2, addr);
}

/* treehash (utils.cu:189-241): stack-based root and auth path */
static void treehash(const hctx *hc, uint8_t *root, uint8_t *auth, uint32_t leaf_idx, uint32_t idx_offset,
                     uint32_t height, gen_leaf_fn gen_leaf, uint8_t tree_addr[32])
{
    const int n = hc->p->n;
    uint8_t *stack = (uint8_t *)malloc((size_t)(height + 1) * n);
    unsigned heights[32];
    unsigned off = 0;
    for (uint32_t idx = 0; idx < (1u << height); idx++) {
        gen_leaf(hc, stack + off * n, idx + idx_offset, tree_addr);
        off++;
        heights[off - 1] = 0;
        if ((leaf_idx ^ 1u) == idx) memcpy(auth, stack + (off - 1) * n, n);
        while (off >= 2 && heights[off - 1] == heights[off - 2]) {
            uint32_t tidx = idx >> (heights[off - 1] + 1);
            set_height(tree_addr, heights[off - 1] + 1);
            set_index(tree_addr, tidx + (idx_offset >> (heights[off - 1] + 1)));
            thash_ctx(hc, stack + (off - 2) * n, stack + (off - 2) * n, 2, tree_addr);
            off--;
            heights[off - 1]++;
            if (((leaf_idx >> heights[off - 1]) ^ 1u) == tidx)
                memcpy(auth + heights[off - 1] * n, stack + (off - 1) * n, n);
        }
    }
    memcpy(root, stack, n);
    free(stack);
}

/* ------------------------------------------------------------------------ */
/* FORS (fors.cu:24-181, 596-632)                                           */
/* ------------------------------------------------------------------------ */

/* fors_gen_leaf (fors.cu:44-56) */
static void fors_gen_leaf(const hctx *hc, uint8_t *leaf, uint32_t addr_idx, const uint8_t tree_addr[32])
{
    uint8_t la[32] = {0};
    copy_keypair(hc->p, la, tree_addr);
    set_type(la, T_FORSTREE);
    set_index(la, addr_idx);
    prf_addr(hc, leaf, la);
    thash_ctx(hc, leaf, leaf, 1, la);
}

/* message_to_indices, LSB-first (fors.cu:77-88) */
static void message_to_indices(const spxo_params *p, uint32_t *idx, const uint8_t *m)
{
    unsigned off = 0;
    for (int i = 0; i < p->k; i++) {
        idx[i] = 0;
        for (int j = 0; j < p->a; j++, off++) idx[i] ^= ((uint32_t)(m[off >> 3] >> (off & 7)) & 1u) << j;
    }
}

/* fors_sign (fors.cu:107-143) */
static void fors_sign(const hctx *hc, uint8_t *sig, uint8_t *pk, const uint8_t *m, const uint8_t fors_addr[32])
{
    const spxo_params *p = hc->p;
    const int n = p->n;
    uint32_t idx[64];
    uint8_t *roots = (uint8_t *)malloc((size_t)p->k * n);
    uint8_t ta[32] = {0}, pa[32] = {0};
    copy_keypair(p, ta, fors_addr);
    copy_keypair(p, pa, fors_addr);
    set_type(ta, T_FORSTREE);
    set_type(pa, T_FORSPK);
    message_to_indices(p, idx, m);
    for (int i = 0; i < p->k; i++) {
        uint32_t off = (uint32_t)i << p->a;
        set_height(ta, 0);
        set_index(ta, idx[i] + off);
        prf_addr(hc, sig, ta);
        sig += n;
        treehash(hc, roots + i * n, sig, idx[i], off, p->a, fors_gen_leaf, ta);
        sig += n * p->a;
    }
    thash_ctx(hc, pk, roots, p->k, pa);
    free(roots);
}

/* fors_pk_from_sig (fors.cu:596-631) */
static void fors_pk_from_sig(const hctx *hc, uint8_t *pk, const uint8_t *sig, const uint8_t *m, const uint8_t fors_addr[32])
{
    const spxo_params *p = hc->p;
    const int n = p->n;
    uint32_t idx[64];
    uint8_t leaf[32];
    uint8_t *roots = (uint8_t *)malloc((size_t)p->k * n);
    uint8_t ta[32] = {0}, pa[32] = {0};
    copy_keypair(p, ta, fors_addr);
    copy_keypair(p, pa, fors_addr);
    set_type(ta, T_FORSTREE);
    set_type(pa, T_FORSPK);
    message_to_indices(p, idx, m);
    for (int i = 0; i < p->k; i++) {
        uint32_t off = (uint32_t)i << p->a;
        set_height(ta, 0);
        set_index(ta, idx[i] + off);
        thash_ctx(hc, leaf, sig, 1, ta);
        sig += n;
        compute_root(hc, roots + i * n, leaf, idx[i], off, sig, p->a, ta);
        sig += n * p->a;
    }
    thash_ctx(hc, pk, roots, p->k, pa);
    free(roots);
}

/* ------------------------------------------------------------------------ */
/* scheme (sign.cu:154-182, 1924-1994, 3048-3121, 3302-3311, 6058-6079)     */
/* ------------------------------------------------------------------------ */

int spxo_seed_keypair(const spxo_params *p, uint8_t *pk, uint8_t *sk, const uint8_t *seed)
{
    const int n = p->n;
    uint8_t auth[16 * 32];
    uint8_t top[32] = {0};
    hctx hc;
    set_layer(top, p->d - 1);
    set_type(top, T_HASHTREE);
    memcpy(sk, seed, 3 * n);
    memcpy(pk, sk + 2 * n, n);
    hctx_init(&hc, p, pk, sk);
    treehash(&hc, sk + 3 * n, auth, 0, 0, p->hp, wots_gen_leaf, top);
    memcpy(pk + n, sk + 3 * n, n);
    return 0;
}

int spxo_sign_signature(const spxo_params *p, uint8_t *sig, size_t *siglen,
                        const uint8_t *m, size_t mlen, const uint8_t *sk, const uint8_t *optrand)
{
    const int n = p->n;
    const uint8_t *sk_seed = sk, *sk_prf = sk + n, *pk = sk + 2 * n, *pub_seed = pk;
    uint8_t mhash[64], root[32];
    uint64_t tree;
    uint32_t idx_leaf;
    uint8_t wa[32] = {0}, ta[32] = {0};
    hctx hc;
    hctx_init(&hc, p, pub_seed, sk_seed);
    set_type(wa, T_WOTS);
    set_type(ta, T_HASHTREE);
    spxo_gen_message_random(p, sig, sk_prf, optrand, m, mlen);
    spxo_hash_message(p, mhash, &tree, &idx_leaf, sig, pk, m, mlen);
    sig += n;
    set_tree(wa, tree);
    set_keypair(p, wa, idx_leaf);
    fors_sign(&hc, sig, root, mhash, wa);
    sig += p->fors_bytes;
    for (int i = 0; i < p->d; i++) {
        set_layer(ta, i);
        set_tree(ta, tree);
        copy_subtree(wa, ta);
        set_keypair(p, wa, idx_leaf);
        wots_sign(&hc, sig, root, wa);
        sig += p->wots_bytes;
        treehash(&hc, root, sig, idx_leaf, 0, p->hp, wots_gen_leaf, ta);
        sig += p->hp * n;
        idx_leaf = (uint32_t)(tree & ((1u << p->hp) - 1));
        tree >>= p->hp;
    }
    if (siglen) *siglen = p->sig_bytes;
    return 0;
}

int spxo_verify(const spxo_params *p, const uint8_t *sig, size_t siglen,
                const uint8_t *m, size_t mlen, const uint8_t *pk)
{
    const int n = p->n;
    const uint8_t *pub_seed = pk, *pub_root = pk + n;
    uint8_t mhash[64], root[32], leaf[32];
    uint8_t wpk[80 * 32];
    uint64_t tree;
    uint32_t idx_leaf;
    uint8_t wa[32] = {0}, ta[32] = {0}, wpa[32] = {0};
    hctx hc;
    if (siglen != (size_t)p->sig_bytes) return -1;
    hctx_init(&hc, p, pub_seed, NULL);
    set_type(wa, T_WOTS);
    set_type(ta, T_HASHTREE);
    set_type(wpa, T_WOTSPK);
    spxo_hash_message(p, mhash, &tree, &idx_leaf, sig, pk, m, mlen);
    sig += n;
    set_tree(wa, tree);
    set_keypair(p, wa, idx_leaf);
    fors_pk_from_sig(&hc, root, sig, mhash, wa);
    sig += p->fors_bytes;
    for (int i = 0; i < p->d; i++) {
        set_layer(ta, i);
        set_tree(ta, tree);
        copy_subtree(wa, ta);
        set_keypair(p, wa, idx_leaf);
        copy_keypair(p, wpa, wa);
        wots_pk_from_sig(&hc, wpk, sig, root, wa);
        sig += p->wots_bytes;
        thash_ctx(&hc, leaf, wpk, p->len, wpa);
        compute_root(&hc, root, leaf, idx_leaf, 0, sig, p->hp, ta);
        sig += p->hp * n;
        idx_leaf = (uint32_t)(tree & ((1u << p->hp) - 1));
        tree >>= p->hp;
    }
    return memcmp(root, pub_root, n) ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* AES-256 (FIPS 197) and the NIST AES-256 CTR DRBG (rng.cu:139-241)        */
/* ------------------------------------------------------------------------ */

static uint8_t SBOX[256];
static int sbox_ready;

static uint8_t gmul(uint8_t a, uint8_t b)
{
    uint8_t r = 0;
    while (b) {
        if (b & 1) r ^= a;
        a = (uint8_t)((a << 1) ^ ((a & 0x80) ? 0x1b : 0));
        b >>= 1;
    }
    return r;
}

/* S-box from its definition: multiplicative inverse in GF(2^8) followed by
 * the affine map b ^ rotl(b,1..4) ^ 0x63 (FIPS 197 section 5.1.1) */
static void aes_tables(void)
{
    if (sbox_ready) return;
    for (int x = 0; x < 256; x++) {
        uint8_t inv = 0;
        if (x) for (int y = 1; y < 256; y++) if (gmul((uint8_t)x, (uint8_t)y) == 1) { inv = (uint8_t)y; break; }
        uint8_t b = inv, s = inv;
        for (int i = 0; i < 4; i++) { b = (uint8_t)((b << 1) | (b >> 7)); s ^= b; }
        SBOX[x] = s ^ 0x63;
    }
    sbox_ready = 1;
}

void spxo_aes256_ecb(const uint8_t key[32], const uint8_t in[16], uint8_t out[16])
{
    uint8_t rk[240];
    uint8_t s[16];
    aes_tables();
    memcpy(rk, key, 32);
    uint8_t rcon = 1;
    for (int i = 8; i < 60; i++) {
        uint8_t t[4];
        memcpy(t, rk + 4 * (i - 1), 4);
        if (i % 8 == 0) {
            uint8_t u = t[0];
            t[0] = SBOX[t[1]] ^ rcon; t[1] = SBOX[t[2]]; t[2] = SBOX[t[3]]; t[3] = SBOX[u];
            rcon = gmul(rcon, 2);
        } else if (i % 8 == 4) {
            for (int j = 0; j < 4; j++) t[j] = SBOX[t[j]];
        }
        for (int j = 0; j < 4; j++) rk[4 * i + j] = rk[4 * (i - 8) + j] ^ t[j];
    }
    for (int i = 0; i < 16; i++) s[i] = in[i] ^ rk[i];
    for (int r = 1; r <= 14; r++) {
        uint8_t t[16];
        for (int i = 0; i < 16; i++) t[i] = SBOX[s[i]];
        /* ShiftRows: row j of column c comes from column c+j */
        for (int c = 0; c < 4; c++)
            for (int j = 0; j < 4; j++) s[4 * c + j] = t[4 * ((c + j) % 4) + j];
        if (r != 14) {
            for (int c = 0; c < 4; c++) {
                uint8_t *col = s + 4 * c, a0 = col[0], a1 = col[1], a2 = col[2], a3 = col[3];
                col[0] = gmul(a0, 2) ^ gmul(a1, 3) ^ a2 ^ a3;
                col[1] = a0 ^ gmul(a1, 2) ^ gmul(a2, 3) ^ a3;
                col[2] = a0 ^ a1 ^ gmul(a2, 2) ^ gmul(a3, 3);
                col[3] = gmul(a0, 3) ^ a1 ^ a2 ^ gmul(a3, 2);
            }
        }
        for (int i = 0; i < 16; i++) s[i] ^= rk[16 * r + i];
    }
    memcpy(out, s, 16);
}

static void v_increment(uint8_t v[16])
{
    for (int j = 15; j >= 0; j--) {
        if (v[j] == 0xff) v[j] = 0;
        else { v[j]++; break; }
    }
}

/* AES256_CTR_DRBG_Update (rng.cu:218-241) */
static void drbg_update(const uint8_t *provided, uint8_t key[32], uint8_t v[16])
{
    uint8_t temp[48];
    for (int i = 0; i < 3; i++) {
        v_increment(v);
        spxo_aes256_ecb(key, v, temp + 16 * i);
    }
    if (provided) for (int i = 0; i < 48; i++) temp[i] ^= provided[i];
    memcpy(key, temp, 32);
    memcpy(v, temp + 32, 16);
}

/* randombytes_init (rng.cu:139-153) */
void spxo_drbg_init(spxo_drbg *s, const uint8_t entropy[48], const uint8_t *personalization)
{
    uint8_t seed[48];
    memcpy(seed, entropy, 48);
    if (personalization) for (int i = 0; i < 48; i++) seed[i] ^= personalization[i];
    memset(s->key, 0, 32);
    memset(s->v, 0, 16);
    drbg_update(seed, s->key, s->v);
    s->reseed_counter = 1;
}

/* randombytes (rng.cu:155-186) */
void spxo_drbg_bytes(spxo_drbg *s, uint8_t *out, size_t len)
{
    uint8_t blk[16];
    while (len > 0) {
        v_increment(s->v);
        spxo_aes256_ecb(s->key, s->v, blk);
        size_t take = len > 15 ? 16 : len;
        memcpy(out, blk, take);
        out += take; len -= take;
    }
    drbg_update(NULL, s->key, s->v);
    s->reseed_counter++;
}

static spxo_drbg g_drbg;
static int g_deterministic = 1;

void spxo_randombytes_init(const uint8_t entropy[48]) { spxo_drbg_init(&g_drbg, entropy, NULL); }
void spxo_randombytes(uint8_t *out, size_t len) { spxo_drbg_bytes(&g_drbg, out, len); }
void spxo_set_deterministic(int on) { g_deterministic = on ? 1 : 0; }

/* crypto_sign_keypair (sign.cu:342-353): draws 3n bytes; under the shipped
 * DEBUG_MODE the seed is then replaced by 0..3n-1 */
int spxo_crypto_sign_keypair(const spxo_params *p, uint8_t *pk, uint8_t *sk)
{
    uint8_t seed[96];
    spxo_randombytes(seed, p->seed_bytes);
    if (g_deterministic) for (int i = 0; i < p->seed_bytes; i++) seed[i] = (uint8_t)i;
    return spxo_seed_keypair(p, pk, sk, seed);
}

/* crypto_sign_signature (sign.cu:1924-1994): draws n bytes of optrand; under
 * DEBUG_MODE it is then replaced by 0xAD bytes (sign.cu:1950-1954) */
int spxo_crypto_sign_signature(const spxo_params *p, uint8_t *sig, size_t *siglen,
                               const uint8_t *m, size_t mlen, const uint8_t *sk)
{
    uint8_t optrand[32];
    spxo_randombytes(optrand, p->n);
    if (g_deterministic) memset(optrand, 0xad, p->n);
    return spxo_sign_signature(p, sig, siglen, m, mlen, sk, optrand);
}

/* crypto_sign (sign.cu:3302-3311) */
int spxo_crypto_sign(const spxo_params *p, uint8_t *sm, unsigned long long *smlen,
                     const uint8_t *m, unsigned long long mlen, const uint8_t *sk)
{
    size_t siglen;
    /* the message may alias sm + sig_bytes; sign from a private copy */
    uint8_t *mc = (uint8_t *)malloc(mlen + 1);
    if (mlen) memcpy(mc, m, mlen);
    spxo_crypto_sign_signature(p, sm, &siglen, mc, (size_t)mlen, sk);
    memmove(sm + p->sig_bytes, mc, mlen);
    free(mc);
    *smlen = siglen + mlen;
    return 0;
}

/* crypto_sign_open (sign.cu:6058-6079) */
int spxo_crypto_sign_open(const spxo_params *p, uint8_t *m, unsigned long long *mlen,
                          const uint8_t *sm, unsigned long long smlen, const uint8_t *pk)
{
    if (smlen < (unsigned long long)p->sig_bytes) {
        memset(m, 0, smlen);
        *mlen = 0;
        return -1;
    }
    *mlen = smlen - p->sig_bytes;
    if (spxo_verify(p, sm, p->sig_bytes, sm + p->sig_bytes, (size_t)*mlen, pk)) {
        memset(m, 0, smlen);
        *mlen = 0;
        return -1;
    }
    memmove(m, sm + p->sig_bytes, *mlen);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* bounded multi-threaded throughput probe (CPU baseline)                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    const spxo_params *p;
    int op, tid;
    size_t mlen;
    double seconds;
    long max_ops;
    long done;
    double elapsed;
} tp_arg;

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static void *tp_worker(void *vp)
{
    tp_arg *a = (tp_arg *)vp;
    const spxo_params *p = a->p;
    uint8_t ent[48], seed[96], pk[64], sk[128], optrand[32];
    spxo_drbg rng;
    for (int i = 0; i < 48; i++) ent[i] = (uint8_t)(i + 97 * a->tid);
    spxo_drbg_init(&rng, ent, NULL);
    spxo_drbg_bytes(&rng, seed, p->seed_bytes);
    spxo_seed_keypair(p, pk, sk, seed);
    uint8_t *m = (uint8_t *)malloc(a->mlen + 1);
    uint8_t *sig = (uint8_t *)malloc(p->sig_bytes);
    spxo_drbg_bytes(&rng, m, a->mlen);
    memset(optrand, 0xad, sizeof(optrand));
    if (a->op == 1) spxo_sign_signature(p, sig, NULL, m, a->mlen, sk, optrand);
    a->done = 0;
    double t0 = now_s(), t = t0;
    while (a->done < a->max_ops) {
        if (a->op == 0) spxo_sign_signature(p, sig, NULL, m, a->mlen, sk, optrand);
        else if (spxo_verify(p, sig, p->sig_bytes, m, a->mlen, pk) != 0) break;
        a->done++;
        t = now_s();
        if (t - t0 >= a->seconds) break;
    }
    a->elapsed = t - t0;
    free(m); free(sig);
    return NULL;
}

long spxo_throughput(const spxo_params *p, int op, int threads, size_t mlen,
                     double min_seconds, long max_ops, double *secs)
{
    if (threads < 1) threads = 1;
    keccak_tables();
    aes_tables();
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    tp_arg *args = (tp_arg *)calloc(threads, sizeof(tp_arg));
    for (int t = 0; t < threads; t++) {
        args[t].p = p; args[t].op = op; args[t].tid = t; args[t].mlen = mlen;
        args[t].seconds = min_seconds; args[t].max_ops = max_ops;
        pthread_create(&th[t], NULL, tp_worker, &args[t]);
    }
    /* aggregate rate = sum of per-worker rates, each timed after its setup;
     * *secs is the equivalent wall time for the total */
    long total = 0;
    double rate = 0;
    for (int t = 0; t < threads; t++) {
        pthread_join(th[t], NULL);
        total += args[t].done;
        if (args[t].elapsed > 0) rate += args[t].done / args[t].elapsed;
    }
    *secs = rate > 0 ? total / rate : 0;
    free(th); free(args);
    return total;
}
