/*
 * cuspx_serve.h -- serving face: a request loop over the batched engine.
 *
 * No counterpart in the reference, whose GPU faces are synchronous calls
 * that allocate, launch and free per batch (sign.cu:5920-5963).  Here
 * requests are admitted as they arrive and continuously batched:
 *   - keys live on the device in a per-set resident table (sk and pk rows);
 *   - requests are split into three message-length classes -- up to
 *     16 KiB, up to 128 KiB, longer -- because message hashing is serial
 *     over the message (a 1 MiB sign hashes for ~33 ms) and a launch ends
 *     with its longest message; one scheduler thread per class groups
 *     pending requests per (operation, set, class) and launches a batch when
 *     the batch is full, the oldest request has waited `window_us`, or no
 *     launch of that group is in flight;
 *   - up to `max_inflight` launches per group run at once on their own
 *     streams (short class at the highest stream priority, long class at the
 *     lowest), so requests arriving while others are on the GPU are admitted
 *     as slots free up and overlap on the device;
 *   - admission by device-memory budget: every request counts the device
 *     bytes its launch will need (scratch plus message) from submission on;
 *     a submission that would take pending plus in-flight bytes over
 *     `mem_budget` is refused with CUSPX_EBUSY, and so is one beyond
 *     `max_queue` pending requests.  The budget thus bounds both the device
 *     memory of in-flight launches and the work queued ahead of a request;
 *   - a launch carries at most 32 MiB of middle-class or 64 MiB of
 *     long-class messages; a single message over 64 MiB is refused with
 *     CUSPX_ETOOBIG;
 *   - per-request latency (submit to result on the host) feeds p50/p99,
 *     overall and per message-length bucket, from fixed log-spaced
 *     histograms (bins 1.1% wide), so memory stays bounded however long the
 *     server runs.
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
    size_t mem_budget;   /* device bytes of pending and in-flight requests (0: 8 GiB) */
    int max_batch;       /* requests per launch (0: 1024) */
    int max_inflight;    /* launches in flight per (operation, set) (0: 3) */
    int window_us;       /* batching window (0: 500 us) */
    int max_keys;        /* resident keys per set (0: 4096) */
    size_t max_queue;    /* pending requests before submit refuses (0: 1<<20) */
    /* Work-based limits (0: off).  A request's GPU work is estimated from its
     * parameter set's hash units (the reference's sign / verify structure)
     * and its message length, in milliseconds of the device's hashing
     * capacity (gpu_ops_per_s).  max_queue_ms refuses a submission with
     * CUSPX_EBUSY when the work pending or in flight would exceed it, which
     * bounds the queueing delay at overload; max_launch_ms caps the work of
     * one launch (at least one request), so a batch of heavy requests
     * (SHAKE-256-256f signs: ~0.1 ms of the whole GPU each) does not keep
     * its group's next requests waiting for long. */
    double max_queue_ms;
    double max_launch_ms;
    double gpu_ops_per_s;   /* integer ops per second the estimates assume (0: 60% of the
                               measured SHA-256-round peak, cuspx_int_peak_mix) */
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
 * returns CUSPX_OK; otherwise returns CUSPX_ETIMEDOUT.  One thread waits on
 * a ticket at a time: a second concurrent wait on it, or a wait on a
 * released or detached ticket, returns CUSPX_EINVAL. */
int cuspx_serve_wait(cuspx_server *s, uint64_t ticket, long timeout_us, uint8_t *sig_out, int32_t *status,
                     double *latency_us);
int cuspx_serve_stats(cuspx_server *s, cuspx_serve_counters *st);
int cuspx_serve_reset_stats(cuspx_server *s);

/* ---- open-loop Poisson load generator ---------------------------------- */
/* one sampled sign request of the load generator (see sample_every) */
typedef struct cuspx_loadgen_sample {
    int32_t set;
    uint32_t key_id;
    int32_t status;   /* the sign request's status */
    uint32_t pad;
    uint64_t mlen, msg_off, sig_off;
} cuspx_loadgen_sample;

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
    /* Sampling of the timed sign requests, so that a caller can check the
     * signatures the stream produced (e.g. against an independent
     * implementation): one sign request in every `sample_every` (0: none)
     * keeps its result, up to `sample_max` samples; sample i's message and
     * signature are copied to arena + samples[i].msg_off / sig_off while
     * arena_bytes last.  The sampled requests are otherwise submitted like
     * the rest (same lengths, sets and timing). */
    uint32_t sample_every;
    uint32_t sample_max;
    cuspx_loadgen_sample *samples;
    uint8_t *arena;
    size_t arena_bytes;
} cuspx_loadgen_config;

typedef struct {
    uint64_t offered, completed, refused, wrong_verdicts, sign_done, verify_done;
    double wall_s, throughput, sign_throughput, verify_throughput;
    double sign_p50_us, sign_p99_us, verify_p50_us, verify_p99_us;
    double mean_batch;
    double sign_p50_bucket_us[3], sign_p99_bucket_us[3], verify_p50_bucket_us[3], verify_p99_bucket_us[3];
    double launch_ms_mean, launch_ms_max;
    /* per entry of cfg->sets (the first 8): completed signs and verifies,
     * and the hash units of their message hashing (SHA-256 compressions or
     * Keccak-f[1600] permutations of PRF_msg and H_msg) */
    uint64_t set_sign_done[8], set_verify_done[8];
    double set_msg_units[8];
    uint64_t sampled;       /* samples written */
} cuspx_loadgen_result;

int cuspx_serve_loadgen(cuspx_server *s, const cuspx_loadgen_config *cfg, cuspx_loadgen_result *out);

#ifdef __cplusplus
}
#endif
#endif
