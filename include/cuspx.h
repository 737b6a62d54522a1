/*
 * cuspx.h -- batched SPHINCS+ engine for one GB300 (sm_103a): C ABI.
 *
 * This is the batched face that sits beside the NIST api.h drop-in
 * (include/spx_api.h).  It replaces the reference's batched GPU launchers
 * with per-item keys, messages of any length, per-item statuses and
 * verdicts:
 *   cuspx_keypair_batch  <- face_mdp_crypto_sign_keypair / face_mhp_crypto_sign_keypair
 *                           (api.h:54-63, sign.cu:1214-1273, :1756-1807)
 *   cuspx_sign_batch     <- face_mdp_crypto_sign / face_mhp_crypto_sign_scheme2
 *                           (api.h:117-131, sign.cu:5098-5195, :5920-5963)
 *   cuspx_verify_batch   <- face_mdp_crypto_sign_open / face_mhp_crypto_sign_open
 *                           (api.h:150-177, sign.cu:6856-6955, :7557-7598)
 * The reference faces fix mlen = 32, use identical keys and return one
 * aggregate verdict; these take per-item keys, lengths and verdicts.
 *
 * Every call returns 0 (CUSPX_OK) or a negative CUSPX_E* code and never
 * aborts; cuspx_error() describes the last failure of a context.
 * Buffers are caller-owned.  Byte layouts follow the reference exactly:
 *   sk  = SK_SEED || SK_PRF || PUB_SEED || ROOT   (4n bytes)
 *   pk  = PUB_SEED || ROOT                         (2n bytes)
 *   sig = R || FORS || d x (WOTS || AUTH)          (cuspx_set_sizes)
 */
#ifndef CUSPX_H
#define CUSPX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUSPX_OK 0
#define CUSPX_EINVAL (-1)     /* bad argument (size, set id, null pointer) */
#define CUSPX_ECUDA (-2)      /* CUDA runtime error, see cuspx_error() */
#define CUSPX_ENOMEM (-3)     /* device memory budget exceeded */
#define CUSPX_EBUSY (-4)      /* queue full / would exceed admission budget */
#define CUSPX_ETIMEDOUT (-5)  /* wait expired */
#define CUSPX_ETOOBIG (-6)    /* request larger than the fixed no-allocation scratch */

enum { CUSPX_OP_KEYGEN = 0, CUSPX_OP_SIGN = 1, CUSPX_OP_VERIFY = 2 };

typedef struct cuspx_ctx cuspx_ctx;
typedef struct cuspx_batch cuspx_batch;

/* ---- parameter sets (params.h:33-79 as a runtime table) --------------- */
int cuspx_num_sets(void);
/* "sha256-128f-simple", "shake256-256f-robust", ...; a bare "sha256-128f"
 * names the simple set.  Returns the set id or CUSPX_EINVAL. */
int cuspx_set_id(const char *name);
const char *cuspx_set_name(int set);
/* sizes in bytes (api.h:12-14, params.h:138-146); any pointer may be null */
int cuspx_set_sizes(int set, size_t *pk_bytes, size_t *sk_bytes, size_t *sig_bytes, size_t *seed_bytes,
                    int *n);

/* ---- context ------------------------------------------------------------ */
int cuspx_create(int device, cuspx_ctx **out);
void cuspx_destroy(cuspx_ctx *ctx);
const char *cuspx_error(const cuspx_ctx *ctx);
/* Launch mapping of one parameter set (the autotuner's output).  Replaces
 * the reference's compile-time knobs (all_option.h:7-68: HP_PARALLELISM,
 * block-size switches, load-balancing switches). */
typedef struct {
    int leaf_block;       /* threads per block, XMSS leaf kernel (multiple of 32) */
    int fors_block;       /* threads per block, FORS kernel (multiple of 32) */
    int verify_block;     /* threads per block, per-item verify kernels (multiple of 32) */
    int tree_warps;       /* warps per block, XMSS tree kernel */
    int chains_per_warp;  /* (item, chain) tasks per warp, verify chain kernel */
    int verify_mode;      /* 0 layered verify kernels, 1 one thread per item over all layers,
                             2 one persistent launch over the whole hypertree (default),
                             3 layered kernels with each layer's WOTS+ chains sorted by length */
    int fors_lanes_log2;  /* lanes per FORS tree = 2^g, g in 0..5 (0: lane per tree, 5: warp per tree) */
    int tree_mode;        /* 0 warp per XMSS subtree, 1 lane per subtree (heights <= 4 only) */
    int chain_mode_max;   /* batches of at most this many signatures (up to 256) compute XMSS
                             leaves one lane per WOTS+ chain instead of one lane per leaf;
                             key generation does so for batches of up to 16384 keys
                             unless this is 0 */
    int verify_slots;     /* most items a warp holds at once in verify_mode 2 (1..8); batches
                             below about 4 warps per SM use fewer */
    int verify_item_max;  /* verify batches of at most this many items (any verify_mode) with one
                             thread block per item: a thread per WOTS+ chain and a T lane that
                             streams T_len behind the chains (0: never) */
    int verify_claim_min; /* verify_mode 2: WOTS+ chains are handed out to free lanes once at
                             least this many lanes of a warp are free (1..32; T streams always
                             at once) */
    int verify_groups;    /* sorted verify: the batch is split into this many groups of items
                             (1..8), each on its own stream, so that one group's serial T_len
                             and auth-path kernel overlaps another group's chains */
    int verify_sorted_min;/* verify batches of at least this many items run the sorted layered
                             verify whatever verify_mode says (0: only with verify_mode 3);
                             batches up to verify_item_max still run one item per block */
    int verify_spec_max;  /* verify batches of at most this many items (0..64; 0: never) first
                             run every WOTS+ chain of every layer from each of its 16 possible
                             start steps in parallel, then walk the layers with T_len and the
                             auth path alone (takes precedence over verify_item_max) */
} cuspx_tuning;
/* fields <= 0 keep the current value, except verify_mode, fors_lanes_log2,
 * tree_mode, chain_mode_max, verify_item_max, verify_sorted_min and
 * verify_spec_max, which keep it when < 0 */
int cuspx_set_tuning(cuspx_ctx *ctx, int set, const cuspx_tuning *t);
int cuspx_get_tuning(cuspx_ctx *ctx, int set, cuspx_tuning *t);
/* Mappings by batch size (what the autotuner installs): the mapping of
 * `set` for `op` batches of min_count..max_count items (inclusive), built
 * from the set's current base mapping with t's fields applied
 * (cuspx_set_tuning's rules).  A batch runs with the entry whose range holds
 * its item count, or with the base mapping if none does.  Ranges of one
 * (set, op) may not overlap (the same range again replaces its entry); at
 * most 16 per (set, op).  Change mappings while no batch of the set is being
 * launched. */
int cuspx_set_tuning_for(cuspx_ctx *ctx, int set, int op, size_t min_count, size_t max_count,
                         const cuspx_tuning *t);
/* the mapping a batch of `count` items of (set, op) runs with */
int cuspx_get_tuning_for(cuspx_ctx *ctx, int set, int op, size_t count, cuspx_tuning *t);
/* drop the entries of (set, op), or of every op when op < 0 */
int cuspx_clear_tuning_for(cuspx_ctx *ctx, int set, int op);
/* Install the entries of a tuning file written by the autotuner
 * (cuspx_gb300/autotune.py): one tab-separated line per entry,
 *   <gpu name> <set name> <sign|verify|keygen> <min_count> <max_count> <ms> <knob>=<v>,...
 * Lines of other GPUs are skipped.  cuspx_create reads $CUSPX_TUNE_CACHE
 * (default $HOME/.cache/cuspx/tune.tsv) when it exists, so the api.h
 * drop-ins, the one-shot calls and serving all run the tuned mappings.
 * Returns the number of entries installed, or a negative error.  Replaces
 * the reference's compile-time launch knobs (all_option.h:7-68). */
int cuspx_load_tuning(cuspx_ctx *ctx, const char *path);
/* the CUDA device name (as the tuning file records it) */
int cuspx_device_name(int device, char *buf, size_t len);

/* ---- one-shot calls on host buffers (synchronous) ----------------------- */
/* seeds: count x 3n; writes pks: count x 2n, sks: count x 4n
 * (crypto_sign_seed_keypair, sign.cu:154-182, per item) */
int cuspx_keypair_batch(cuspx_ctx *ctx, int set, size_t count, const uint8_t *seeds, uint8_t *pks, uint8_t *sks);
/* sks: count x 4n rows; message i is msgs[msg_off[i] .. +msg_len[i]);
 * optrand: count x n or NULL for the reference's fixed 0xAD bytes
 * (sign.cu:1950-1954); sigs: count x sig_bytes; status[i] = 0 on success,
 * -2 if the key's ROOT does not match its seeds (may be NULL). */
int cuspx_sign_batch(cuspx_ctx *ctx, int set, size_t count, const uint8_t *sks, const uint8_t *msgs,
                     const uint64_t *msg_off, const uint64_t *msg_len, const uint8_t *optrand, uint8_t *sigs,
                     int32_t *status);
/* pks: count x 2n rows; sigs: count rows of sig_bytes; siglens: per item
 * (NULL = sig_bytes).  verdicts[i] = 0 accept, -1 reject
 * (crypto_sign_verify, sign.cu:3048-3121); -3 if the per-item verify kernel
 * (cuspx_tuning.verify_item_max) gave up waiting for its own chain threads,
 * which its design never lets happen (the wait is bounded all the same). */
int cuspx_verify_batch(cuspx_ctx *ctx, int set, size_t count, const uint8_t *pks, const uint8_t *msgs,
                       const uint64_t *msg_off, const uint64_t *msg_len, const uint8_t *sigs,
                       const uint64_t *siglens, int32_t *verdicts);

/* ---- reusable device-resident batches ----------------------------------
 * A batch owns device buffers for up to `capacity` items of one op and set,
 * its own CUDA stream and a CUDA graph of its launch sequence (captured on
 * the first run of each item count).  upload/run/download are asynchronous
 * on that stream; download and sync wait.  Message offsets passed to upload
 * must be multiples of 16. */
int cuspx_batch_create(cuspx_ctx *ctx, int op, int set, size_t capacity, size_t msg_capacity, size_t key_capacity,
                       cuspx_batch **out);
void cuspx_batch_destroy(cuspx_batch *b);
/* keys: nkeys rows (sk for keygen/sign -- keygen rows carry the seed in
 * their first 3n bytes -- pk for verify); key_index: per item row, or NULL
 * for row i.  aux: sign -> optrand (count x n) or NULL; verify -> sigs
 * (count x sig_bytes); siglens: verify only, may be NULL. */
int cuspx_batch_upload(cuspx_batch *b, size_t count, const uint8_t *keys, size_t nkeys, const uint32_t *key_index,
                       const uint8_t *msgs, size_t msg_bytes, const uint64_t *msg_off, const uint64_t *msg_len,
                       const uint8_t *aux, const uint64_t *siglens);
int cuspx_batch_run(cuspx_batch *b);
/* sign -> out = sigs; verify -> out unused (verdicts in status);
 * keygen -> out = sk rows, out2 = pk rows */
int cuspx_batch_download(cuspx_batch *b, uint8_t *out, uint8_t *out2, int32_t *status);
/* same copies, enqueued on the batch stream without waiting (host buffers
 * must be pinned for the copies to overlap; completion by cuspx_batch_sync
 * or an event recorded on cuspx_batch_stream) */
int cuspx_batch_download_async(cuspx_batch *b, uint8_t *out, uint8_t *out2, int32_t *status);
int cuspx_batch_sync(cuspx_batch *b);
/* device time of the last run, from CUDA events recorded on the batch stream */
int cuspx_batch_last_ms(cuspx_batch *b, float *ms);
/* the batch's cudaStream_t */
void *cuspx_batch_stream(cuspx_batch *b);
/* Use a device-resident key table (nkeys rows of sk for sign, pk for verify,
 * owned by the caller and kept alive while the batch uses it) instead of
 * uploading keys; upload() is then called with keys = NULL and a key_index.
 * Pass d_keys = NULL to unbind. */
int cuspx_batch_bind_keys(cuspx_batch *b, const void *d_keys, size_t nkeys);
/* device pointers of the batch buffers (for device-resident callers) */
int cuspx_batch_device_ptrs(cuspx_batch *b, void **keys, void **msgs, void **msg_off, void **msg_len, void **aux,
                            void **out, void **status);
/* per-kernel timing: when enabled, run() launches without the graph and
 * records an event pair around every kernel; cuspx_batch_kernel_ms returns
 * the names and accumulated milliseconds (count entries). */
int cuspx_batch_profile(cuspx_batch *b, int enable);
int cuspx_batch_kernel_ms(cuspx_batch *b, int idx, const char **name, double *ms, long *launches);

/* ---- mixed parameter sets in one launch ---------------------------------
 * Runs the launch sequences of nb uploaded batches (any ops and sets of this
 * context) as ONE CUDA graph: the graph forks onto every batch's stream so
 * different parameter sets execute concurrently, and joins at the end.  The
 * graph is captured on first use of a given (batches, counts, tunings)
 * combination and replayed afterwards.  Synchronous; *ms (may be NULL)
 * receives the device time of the whole graph.  Results are read with
 * cuspx_batch_download on each batch. */
int cuspx_group_run(cuspx_ctx *ctx, cuspx_batch *const *batches, int nb, float *ms);

/* ---- signing without device allocation ----------------------------------
 * No counterpart in the reference (whose GPU faces cudaMalloc and cudaFree on
 * every call).  For callers that must not allocate device memory while they
 * run: cudaFree waits for the whole device and stalls every other stream,
 * and hosts that own all device memory through their own allocator forbid a
 * library from allocating.  The caller passes DEVICE pointers for all inputs
 * and outputs (same layouts as cuspx_sign_batch: count sk rows of 4n bytes;
 * a message slab with 16-byte aligned offsets, readable up to the next
 * multiple of 16 past each message; optrand count x n or NULL for the
 * reference's 0xAD bytes; count x sig_bytes signatures; count statuses) and
 * the cudaStream_t to run on (NULL: legacy default stream).
 *   - Alignment: d_msgs must be 16-byte aligned; d_sks, d_optrand, d_sigs,
 *     d_msg_off and d_msg_len 8-byte aligned; d_status 4-byte aligned.
 *     Otherwise CUSPX_EINVAL is returned and nothing is launched.  The
 *     per-item offsets live on the device and cannot be checked: each must
 *     be a multiple of 16.  d_msgs must not be NULL, even when every
 *     message is empty (the lengths are not visible to the host).
 * The call is asynchronous on that stream and allocates nothing: its scratch is an
 * 8 MiB array in the library's device image, held by every GPU that loads
 * the library until the process exits.
 *   - Limit: count must fit the 8 MiB scratch; the per-signature need is
 *     d*len*16*n + d*2^h'*n + d*n + k*n + 96 bytes (about 196 KiB at 128f:
 *     41 signatures; 118 KiB at 128s: 69; 426 KiB at 192f: 19; 580 KiB at
 *     256f: 14).  Larger batches return CUSPX_ETOOBIG and launch nothing.
 *   - The first call on a device (with that device current) resolves the
 *     array's device address and configures the kernels; make that first
 *     call before any stream capture.
 *   - Every call shares the array: calls that overlap on the GPU race and
 *     must be serialised by the caller.  It is never cleared; no scratch
 *     value is read before the same call writes it. */
int cuspx_sign_noalloc(int set, size_t count, const uint8_t *d_sks, const uint8_t *d_msgs,
                       const uint64_t *d_msg_off, const uint64_t *d_msg_len, const uint8_t *d_optrand,
                       uint8_t *d_sigs, int32_t *d_status, void *stream);

/* ---- calibration --------------------------------------------------------
 * Measured integer peak of this GPU on all SMs at full occupancy: the
 * roofline denominator for the hash kernels.  mix 0: ALU pipe alone
 * (funnel-shift rotate, 3-input logic, 3-input add; the Keccak-f shape);
 * mix 1: a SHA-256 round as the hash core issues it, 7 ALU ops to one add
 * on the FMA pipe.  cuspx_int_peak is mix 0.  No counterpart in the
 * reference, which publishes no roofline. */
int cuspx_int_peak_mix(int device, int iters, int mix, double *ops_per_s, float *ms);
int cuspx_int_peak(int device, int iters, double *ops_per_s, float *ms);
/* SHA-256 compressions per second over all SMs, with warps_per_sm warps on
 * every SM, each lane running `iters` compressions in a dependent chain (each
 * block built from the previous state); *ns_per_cmp (may be NULL) is the
 * time of one compression in such a chain.  At one warp per SM this is the
 * compression's latency, the floor of a serial hash path. */
int cuspx_cmp_rate(int device, int warps_per_sm, int iters, double *cmp_per_s, double *ns_per_cmp);

#ifdef __cplusplus
}
#endif
#endif
