/*
 * spx_api.h -- NIST signature API, the drop-in replacement for the
 * reference's api.h (api.h:19-136) and rng.h (rng.h:48-55).
 *
 * One shared library per parameter set, libspx_<set>.so (for example
 * libspx_sha256-128f-simple.so), exports exactly these names with the
 * reference's semantics; the work runs on the GPU through libcuspx.so.
 * The set is fixed when the library is built, as the reference fixes it
 * with -D flags (Makefile:109-155).
 *
 * Conventions (sign.cu:3048-3121, :6058-6079):
 *   - return 0 on success; verify/open return -1 on any failure;
 *   - crypto_sign_open zero-fills m over smlen bytes and sets *mlen = 0 on
 *     failure; sm = sig || m; in-place open (m == sm) is allowed;
 *   - crypto_sign_keypair draws 3n bytes and crypto_sign_signature n bytes
 *     from the process-global DRBG, in that order, like the reference.
 * Unlike the reference these calls are thread-safe.
 */
#ifndef SPX_API_H
#define SPX_API_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
#define CRYPTO_ALGNAME "SPHINCS+"

/* sign.cu:124-147 */
unsigned long long crypto_sign_secretkeybytes(void);
unsigned long long crypto_sign_publickeybytes(void);
unsigned long long crypto_sign_bytes(void);
unsigned long long crypto_sign_seedbytes(void);

/* sign.cu:154 -- sk = SK_SEED || SK_PRF || PUB_SEED || ROOT, pk = PUB_SEED || ROOT */
int crypto_sign_seed_keypair(unsigned char *pk, unsigned char *sk, const unsigned char *seed);
/* sign.cu:342 */
int crypto_sign_keypair(unsigned char *pk, unsigned char *sk);
/* sign.cu:1924 */
int crypto_sign_signature(uint8_t *sig, size_t *siglen, const uint8_t *m, size_t mlen, const uint8_t *sk);
/* sign.cu:3048 */
int crypto_sign_verify(const uint8_t *sig, size_t siglen, const uint8_t *m, size_t mlen, const uint8_t *pk);
/* sign.cu:3302 */
int crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m, unsigned long long mlen,
                const unsigned char *sk);
/* sign.cu:6058 */
int crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm, unsigned long long smlen,
                     const unsigned char *pk);

/* rng.h:48-55 */
void randombytes_init(unsigned char *entropy_input, unsigned char *personalization_string, int security_strength);
int randombytes(unsigned char *x, unsigned long long xlen);

/*
 * The reference's GPU faces (api.h:49-176), same names and buffer layouts.
 * The variants differ in the reference only by their parallel scheme ("ap"
 * algorithmic, "dp/mdp/sdp" thread per signature, "mhp" hybrid with
 * intra_para threads, "ms" multi-stream, "mgpu" two devices); here every
 * variant is the same batched GPU engine with the autotuned mapping, so
 * intra_para is accepted and ignored.  Unlike the reference they compute
 * exactly the CPU path's bytes (optrand 0xAD..., sign.cu:1951-1954) and
 * verify every item (the reference's batched open reports task 0 only).
 *   single:  face_crypto_sign_keypair / face_crypto_sign / face_crypto_sign_open
 *            (and the face_ap_* aliases)
 *   batched: sk/pk are num rows; m is num messages of mlen bytes each; sm is
 *            num rows of (sig || m_i), smlen the length of one row; open
 *            writes num messages of smlen - CRYPTO_BYTES bytes into m,
 *            zero-filling the rows that fail, and returns 0 only if every
 *            item verified (else -1).
 */
int face_crypto_sign_keypair(unsigned char *pk, unsigned char *sk);
int face_ap_crypto_sign_keypair(unsigned char *pk, unsigned char *sk);
int face_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m, unsigned long long mlen,
                     const unsigned char *sk);
int face_ap_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                        unsigned long long mlen, const unsigned char *sk);
int face_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                          unsigned long long smlen, const unsigned char *pk);
int face_ap_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                             unsigned long long smlen, const unsigned char *pk);
int face_mdp_crypto_sign_keypair(unsigned char *pk, unsigned char *sk, unsigned int num);
int face_mhp_crypto_sign_keypair(unsigned char *pk, unsigned char *sk, unsigned int num, unsigned int intra_para);
int face_mhp_crypto_sign_keypair_scheme2(unsigned char *pk, unsigned char *sk, unsigned int num,
                                         unsigned int intra_para);
int face_mdp_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                         unsigned long long mlen, const unsigned char *sk, unsigned int dp_num);
int face_sdp_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                         unsigned long long mlen, const unsigned char *sk, unsigned int dp_num);
int face_mhp_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                         unsigned long long mlen, const unsigned char *sk, unsigned int dp_num);
int face_mhp_crypto_sign_scheme2(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                                 unsigned long long mlen, const unsigned char *sk, unsigned int dp_num,
                                 unsigned int intra_para);
int face_mdp_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                              unsigned long long smlen, const unsigned char *pk, unsigned int dp_num);
int face_sdp_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                              unsigned long long smlen, const unsigned char *pk, unsigned int dp_num);
int face_mhp_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                              unsigned long long smlen, const unsigned char *pk, unsigned int dp_num,
                              unsigned int intra_para);

#ifdef __cplusplus
}
#endif
#endif
