/*
 * cuspx_serve.h -- serving face: a request loop over the batched engine.
 *
 * No counterpart in the reference, whose GPU faces are synchronous calls
 * that allocate, launch and free per batch (sign.cu:5920-5963).  Here
 * requests are admitted as they arrive and continuously batched:
 *   - keys live on the device in a per-set resident table (sk and pk rows);
 *   - scheduler threads (one for messages up to 16 KiB, one for longer
 *     ones) group pending requests per (operation, set, length class) and
 *     launch a batch when the batch is full, the oldest request has waited
 *     `window_us`, or no launch of that group is in flight;
 *   - up to `max_inflight` launches per group run at once on their own
 *     streams, so requests arriving while others are on the GPU are admitted
 *     as slots free up and overlap on the device;
 *   - a launch is admitted only while the device bytes of all in-flight
 *     launches stay within `mem_budget`; submissions beyond `max_queue`
 *     pending requests are refused with CUSPX_EBUSY;
 *   - requests with messages over 16 KiB are batched apart from shorter ones
 *     (their serial message hashing would hold a shared batch back); a
 *     launch carries at most 64 MiB of long messages, and a single message
 *     over 64 MiB is refused with CUSPX_ETOOBIG;
 *   - per-request latency (submit to result on the host) feeds p50/p99,
 *     overall and per message-length bucket.
 * Results of a request do not depend on what it was batched with.
 */
#ifndef CUSPX_SERVE_H
#define CUSPX_SERVE_H

#include <stddef.h>
#include <stdint.h>

#include "cuspx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cuspx_server cuspx_server;

typedef struct {
    size_t mem_budget;   /* device bytes for in-flight launches (0: 8 GiB) */
    int max_batch;       /* requests per launch (0: 1024) */
    int max_inflight;    /* launches in flight per (operation, set) (0: 3) */
    int window_us;       /* batching window (0: 500 us) */
    int max_keys;        /* resident keys per set (0: 4096) */
    size_t max_queue;    /* pending requests before submit refuses (0: 1<<20) */
} cuspx_serve_config;

typedef struct {
    uint64_t submitted, completed, refused, failed, launches;
    uint64_t sign_done, verify_done;
    size_t bytes_inflight, bytes_peak;
    double sign_p50_us, sign_p99_us, verify_p50_us, verify_p99_us;
    double mean_batch;
    /* latency by message length: [0] <= 1 KiB, [1] <= 64 KiB, [2] > 64 KiB */
    double sign_p50_bucket_us[3], sign_p99_bucket_us[3], verify_p50_bucket_us[3], verify_p99_bucket_us[3];
    uint64_t bucket_count[2][3];   /* [sign, verify][bucket] */
    double launch_ms_mean, launch_ms_max;   /* device time of a launch: upload + kernels + download */
} cuspx_serve_counters;

/* submit flags */
#define CUSPX_SUBMIT_BORROW 1u   /* msg/sig stay valid until completion: no copy at submit */
#define CUSPX_SUBMIT_DETACH 2u   /* nobody waits: the request is released at completion */

int cuspx_serve_create(cuspx_ctx *ctx, const cuspx_serve_config *cfg, cuspx_server **out);
/* stops admission, waits (bounded) for in-flight launches and frees everything */
void cuspx_serve_destroy(cuspx_server *s);
/* resident keys: count secret keys (4n bytes each) of `set`; ids are
 * consecutive from *first_id.  The public key of each is its sk[2n..4n). */
int cuspx_serve_add_keys(cuspx_server *s, int set, size_t count, const uint8_t *sks, uint32_t *first_id);
/* Create every launch slot of (op, set) now -- the device batch and pinned
 * staging of up to max_inflight launches for each message-length class --
 * instead of when the first requests need them, so that no allocation falls
 * on the serving path (device allocation can wait for the GPU).  Optional;
 * no counterpart in the reference, whose GPU faces allocate per call. */
int cuspx_serve_prepare(cuspx_server *s, int op, int set);
/* public-only keys for verification (2n bytes each); signing with them fails */
int cuspx_serve_add_pubkeys(cuspx_server *s, int set, size_t count, const uint8_t *pks, uint32_t *first_id);
/* op: CUSPX_OP_SIGN (sig ignored) or CUSPX_OP_VERIFY (sig/siglen checked) */
int cuspx_serve_submit(cuspx_server *s, int op, int set, uint32_t key_id, const uint8_t *msg, size_t mlen,
                       const uint8_t *sig, size_t siglen, unsigned flags, uint64_t *ticket);
/* Wait up to timeout_us (< 0: forever) for a request.  On completion copies
 * the signature (sign) into sig_out if not NULL, the status (sign: 0 or
 * <0; verify: 0 accept / -1 reject) and latency, releases the ticket and
 * returns CUSPX_OK; otherwise returns CUSPX_ETIMEDOUT. */
int cuspx_serve_wait(cuspx_server *s, uint64_t ticket, long timeout_us, uint8_t *sig_out, int32_t *status,
                     double *latency_us);
int cuspx_serve_stats(cuspx_server *s, cuspx_serve_counters *st);
int cuspx_serve_reset_stats(cuspx_server *s);

/* ---- open-loop Poisson load generator ---------------------------------- */
typedef struct {
    double rate;            /* arrivals per second */
    double seconds;         /* length of the arrival window */
    double verify_frac;     /* share of verify requests */
    int nsets;
    const int *sets;        /* parameter sets, drawn uniformly */
    uint32_t keys_per_set;  /* keys 0..keys_per_set-1 of each set must be resident */
    uint64_t min_len, max_len;  /* message length, log-uniform */
    double corrupt_frac;    /* verify requests with one seeded byte flipped */
    uint64_t seed;
    int pool;               /* pre-signed (message, signature) pairs per set for verify */
} cuspx_loadgen_config;

typedef struct {
    uint64_t offered, completed, refused, wrong_verdicts, sign_done, verify_done;
    double wall_s, throughput, sign_throughput, verify_throughput;
    double sign_p50_us, sign_p99_us, verify_p50_us, verify_p99_us;
    double mean_batch;
    double sign_p50_bucket_us[3], sign_p99_bucket_us[3], verify_p50_bucket_us[3], verify_p99_bucket_us[3];
    double launch_ms_mean, launch_ms_max;
} cuspx_loadgen_result;

int cuspx_serve_loadgen(cuspx_server *s, const cuspx_loadgen_config *cfg, cuspx_loadgen_result *out);

#ifdef __cplusplus
}
#endif
#endif
