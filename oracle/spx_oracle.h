/*
 * spx_oracle.h -- CPU restatement of the reference SPHINCS+ path (TEST
 * INFRASTRUCTURE ONLY).
 *
 * This is the checker the GPU engine is compared against.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline legs may load it; the
 * product library never links or calls it.
 *
 * Parity pin: the simple SHA-256 and SHAKE-256 sets are pinned byte-for-byte
 * against the reference's own CPU code (sign.cu / wots.cu / fors.cu /
 * utils.cu / sha256.cu / fips202.cu, compiled by oracle/build_ref.sh) through
 * the fixtures in tests/golden.  The robust sets do not exist in the
 * reference: for them parity is UNPINNED -- the tweakable hash follows the
 * published SPHINCS+ round-3 robust construction on top of the reference's
 * own hash, ADRS layout and message hashing.
 *
 * Unlike the reference (process-global state_seeded, DRBG_ctx) every call
 * here is re-entrant: hash state lives in an explicit context.
 */
#ifndef SPX_ORACLE_H
#define SPX_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { SPXO_SHA256 = 0, SPXO_SHAKE256 = 1 };

/* Runtime parameter descriptor; the reference fixes these at compile time
 * (params.h:33-146). */
typedef struct {
    int hash;    /* SPXO_SHA256 or SPXO_SHAKE256 */
    int robust;  /* 0 simple, 1 robust */
    int n, h, d, a, k, w;
    /* derived */
    int hp;             /* tree height h/d */
    int len1, len2, len;/* WOTS chain counts */
    int fors_msg_bytes; /* ceil(a*k/8) */
    int fors_bytes;     /* (a+1)*k*n */
    int wots_bytes;     /* len*n */
    int sig_bytes, pk_bytes, sk_bytes, seed_bytes;
    int tree_bits, tree_bytes, leaf_bits, leaf_bytes, dgst_bytes;
} spxo_params;

/* Fills *p from a name such as "sha256-128f-simple" or "shake256-256f-robust".
 * Returns 0 on success, -1 for an unknown name. */
int spxo_params_from_name(spxo_params *p, const char *name);
/* Fills *p from explicit values (w must be 16); returns 0 or -1. */
int spxo_params_init(spxo_params *p, int hash, int robust, int n, int h, int d, int a, int k);

/* NIST API, re-entrant, over an explicit parameter set.  The deterministic
 * flag reproduces the reference's unconditional DEBUG_MODE (all_option.h:75):
 * keypair seeds are forced to 0..3n-1 and optrand to 0xAD after the DRBG has
 * been drawn. */
int spxo_seed_keypair(const spxo_params *p, uint8_t *pk, uint8_t *sk, const uint8_t *seed);
int spxo_sign_signature(const spxo_params *p, uint8_t *sig, size_t *siglen,
                        const uint8_t *m, size_t mlen, const uint8_t *sk, const uint8_t *optrand);
int spxo_verify(const spxo_params *p, const uint8_t *sig, size_t siglen,
                const uint8_t *m, size_t mlen, const uint8_t *pk);

/* Reference-API mirrors with the process-global DRBG (sign.cu:342, :1924,
 * :3302, :6058). */
void spxo_set_deterministic(int on);
int spxo_crypto_sign_keypair(const spxo_params *p, uint8_t *pk, uint8_t *sk);
int spxo_crypto_sign_signature(const spxo_params *p, uint8_t *sig, size_t *siglen,
                               const uint8_t *m, size_t mlen, const uint8_t *sk);
int spxo_crypto_sign(const spxo_params *p, uint8_t *sm, unsigned long long *smlen,
                     const uint8_t *m, unsigned long long mlen, const uint8_t *sk);
int spxo_crypto_sign_open(const spxo_params *p, uint8_t *m, unsigned long long *mlen,
                          const uint8_t *sm, unsigned long long smlen, const uint8_t *pk);

/* Pieces exposed for unit tests. */
void spxo_sha256(uint8_t out[32], const uint8_t *in, size_t inlen);
void spxo_shake256(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen);
void spxo_mgf1(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen);
void spxo_aes256_ecb(const uint8_t key[32], const uint8_t in[16], uint8_t out[16]);
void spxo_thash(const spxo_params *p, uint8_t *out, const uint8_t *in, unsigned inblocks,
                const uint8_t *pub_seed, const uint8_t addr[32]);
void spxo_hash_message(const spxo_params *p, uint8_t *digest, uint64_t *tree, uint32_t *leaf_idx,
                       const uint8_t *R, const uint8_t *pk, const uint8_t *m, size_t mlen);
void spxo_gen_message_random(const spxo_params *p, uint8_t *R, const uint8_t *sk_prf,
                             const uint8_t *optrand, const uint8_t *m, size_t mlen);

/* AES-256 CTR DRBG (rng.cu:139-241), explicit-state and process-global forms. */
typedef struct { uint8_t key[32]; uint8_t v[16]; int reseed_counter; } spxo_drbg;
void spxo_drbg_init(spxo_drbg *s, const uint8_t entropy[48], const uint8_t *personalization);
void spxo_drbg_bytes(spxo_drbg *s, uint8_t *out, size_t len);
void spxo_randombytes_init(const uint8_t entropy[48]);
void spxo_randombytes(uint8_t *out, size_t len);

/* Hash units counted on the calling thread since spxo_units_reset:
 * out[0] SHA-256 compressions, out[1] Keccak-f[1600] permutations, out[2]
 * the units of both inside wots_sign (wots.cu:614-625). */
void spxo_units(unsigned long long out[3]);
void spxo_units_reset(void);

/* Bounded multi-threaded throughput probe used by the CPU baseline: each of
 * `threads` workers signs (op=0) or verifies (op=1) its share of `count`
 * items with distinct seeded keys for at least `min_seconds`.  Returns the
 * number of operations completed and the wall seconds taken in *secs. */
long spxo_throughput(const spxo_params *p, int op, int threads, size_t mlen,
                     double min_seconds, long max_ops, double *secs);

#ifdef __cplusplus
}
#endif
#endif
