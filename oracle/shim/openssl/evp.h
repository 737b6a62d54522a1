/* Prototype-only stand-in for the four libcrypto entry points the reference
 * DRBG calls (AES-256-ECB through the EVP interface).  The oracle build links
 * the real system libcrypto.so.3; this header only declares what it needs
 * because the OpenSSL development headers are not installed here. */
#ifndef CUSPX_SHIM_OPENSSL_EVP_H
#define CUSPX_SHIM_OPENSSL_EVP_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct evp_cipher_ctx_st EVP_CIPHER_CTX;
typedef struct evp_cipher_st EVP_CIPHER;
typedef struct engine_st ENGINE;
EVP_CIPHER_CTX *EVP_CIPHER_CTX_new(void);
void EVP_CIPHER_CTX_free(EVP_CIPHER_CTX *c);
const EVP_CIPHER *EVP_aes_256_ecb(void);
int EVP_EncryptInit_ex(EVP_CIPHER_CTX *ctx, const EVP_CIPHER *cipher, ENGINE *impl,
                       const unsigned char *key, const unsigned char *iv);
int EVP_EncryptUpdate(EVP_CIPHER_CTX *ctx, unsigned char *out, int *outl,
                      const unsigned char *in, int inl);
#ifdef __cplusplus
}
#endif
#endif
