// engine.cu -- host engine behind include/cuspx.h.
//
// Owns contexts (one device each), reusable device-resident batches with
// their own stream and CUDA graph, and the one-shot host-buffer calls.  The
// reference's equivalents (face_* launchers in sign.cu) cudaMalloc, copy,
// launch cooperatively, synchronise and free on every call; here buffers
// persist per batch and the launch sequence is a replayed CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cuspx.h"
#include "spx_launch.cuh"
#include "spx_sets.h"

namespace cuspx {
FamilyOps g_family[2][3][2];
void register_family_0_16_0();
void register_family_0_16_1();
void register_family_0_24_0();
void register_family_0_24_1();
void register_family_0_32_0();
void register_family_0_32_1();
void register_family_1_16_0();
void register_family_1_16_1();
void register_family_1_24_0();
void register_family_1_24_1();
void register_family_1_32_0();
void register_family_1_32_1();

static std::once_flag g_reg_once;
static void register_all() {
    std::call_once(g_reg_once, [] {
        register_family_0_16_0(); register_family_0_16_1();
        register_family_0_24_0(); register_family_0_24_1();
        register_family_0_32_0(); register_family_0_32_1();
        register_family_1_16_0(); register_family_1_16_1();
        register_family_1_24_0(); register_family_1_24_1();
        register_family_1_32_0(); register_family_1_32_1();
    });
}

SetParams make_params(const SetDesc &s) {
    SetParams P;
    P.n = s.n; P.h = s.h; P.d = s.d; P.hp = s.h / s.d; P.a = s.a; P.k = s.k;
    P.len1 = 2 * s.n;
    P.len2 = 3;
    P.len = P.len1 + P.len2;
    P.fors_msg_bytes = (s.a * s.k + 7) / 8;
    P.fors_bytes = (s.a + 1) * s.k * s.n;
    P.wots_bytes = P.len * s.n;
    P.sig_bytes = s.n + P.fors_bytes + s.d * P.wots_bytes + s.h * s.n;
    P.tree_bits = P.hp * (s.d - 1);
    P.tree_bytes = (P.tree_bits + 7) / 8;
    P.leaf_bits = P.hp;
    P.leaf_bytes = (P.leaf_bits + 7) / 8;
    P.dgst_bytes = P.fors_msg_bytes + P.tree_bytes + P.leaf_bytes;
    P.pk_bytes = 2 * s.n;
    P.sk_bytes = 4 * s.n;
    return P;
}

static const FamilyOps &family_of(int set) {
    const SetDesc &s = kSets[set];
    return g_family[s.hash][s.n / 8 - 2][s.robust];
}

// registration for other translation units of the library
void ensure_registered() { register_all(); }
}  // namespace cuspx

using namespace cuspx;

// items per batch for which chain-parallel leaf scratch is allocated (the
// largest chain_mode_max that can take effect)
static const size_t kChainModeItems = 256;
// items per verify batch that the speculative chain table covers (the
// largest verify_spec_max; 64 x 22 x 35 x 16 x 16 B = 12.6 MB at 128f)
static const int kSpecItems = 64;
// keys per key-generation batch that the chain-parallel scratch covers
// (16384 x 2^hp x len x n: 73 MB at 128f)
static const size_t kKeygenChainItems = 16384;
// messages of at least this many bytes (32 SHA-256 blocks) are hashed by the
// two-warp message kernels of the SHA-256 sets
static const uint64_t kPairMsgBytes = 2048;

struct OneshotJob;

// a tuned mapping for batches of min_count..max_count items of one (set, op)
struct TuneEntry {
    size_t min_count, max_count;
    Tuning t;
};
constexpr int kMaxTuneEntries = 16;

struct cuspx_ctx {
    int device = 0;
    std::mutex err_mu;   // err is written by any calling thread
    std::string err;
    Tuning tune[kNumSets];
    // per-size entries (sorted by min_count) that take precedence over tune[]
    TuneEntry tune_for[kNumSets][3][kMaxTuneEntries];
    int ntune_for[kNumSets][3] = {};
    bool configured[2][3][2] = {};
    // one-shot calls: queued jobs and whether a caller is running a launch
    std::mutex comb_mu;
    std::condition_variable comb_cv;
    std::deque<OneshotJob *> comb_q;
    bool comb_busy = false;
    std::mutex mu;       // one-shot batches
    std::mutex cfg_mu;   // kernel attribute configuration
    cuspx_batch *oneshot[3][kNumSets] = {};
    uint8_t *stage = nullptr;   // pinned staging of the one-shot calls (under mu)
    size_t stage_cap = 0;
    // multi-batch (mixed parameter set) graphs
    struct GroupGraph {
        std::vector<cuspx_batch *> batches;
        std::vector<size_t> counts;
        std::vector<bool> long_msgs;
        std::vector<Tuning> tunes;
        cudaGraphExec_t exec;
        cudaStream_t origin;
        cudaEvent_t e0, e1;
    };
    std::vector<GroupGraph> groups;
    std::mutex group_mu;
};

struct ProfEntry {
    const char *name;
    double ms;
    long launches;
};

struct cuspx_batch {
    cuspx_ctx *ctx = nullptr;
    int op = 0, set = 0;
    SetParams P{};
    size_t cap = 0, msg_cap = 0, key_cap = 0;
    cudaStream_t s = nullptr;
    bool own_stream = true;    // false: s belongs to the caller (batch_share_stream)
    StreamFork fork{};         // sign batches: FORS beside the hypertree
    uint8_t *keys = nullptr;
    uint32_t *keyrow = nullptr;
    uint8_t *msg = nullptr;
    uint64_t *off = nullptr, *len = nullptr;
    uint8_t *aux = nullptr;
    uint64_t *siglen = nullptr;
    uint8_t *out = nullptr;
    int32_t *status = nullptr;
    SignWork *work = nullptr;
    uint8_t *fors_roots = nullptr, *leaves = nullptr, *roots = nullptr, *chains = nullptr;
    uint8_t *wpk = nullptr, *cur_root = nullptr;
    uint32_t *ctr = nullptr;   // persistent verify item counter
    VerifyLists vlists{};      // verify_mode 3: chains bucketed by steps
    VerifyFork vfork{};        // verify_mode 3: streams of the item groups
    bool long_msgs = false;    // the last upload held a message of >= kPairMsgBytes (SHA-256:
                               // hash those over two warps; both kernels read the device
                               // lengths, so the split is right whatever the flag says)
    uint8_t *ends = nullptr;   // chain-parallel leaf scratch
    uint32_t ends_cap = 0;
    size_t count = 0;
    bool use_keyrow = false, use_aux = false, use_siglen = false;
    const uint8_t *bound_keys = nullptr;   // external device key table (not owned)
    size_t bound_nkeys = 0;
    // captured launch sequences keyed by everything baked into them; an item
    // count seen for the first time launches directly and is captured on
    // its second use
    struct GraphKey {
        size_t count;
        bool keyrow, aux, siglen, long_msgs;
        const uint8_t *keys;
        Tuning tune;
        bool operator==(const GraphKey &o) const {
            return count == o.count && keyrow == o.keyrow && aux == o.aux && siglen == o.siglen &&
                   long_msgs == o.long_msgs && keys == o.keys && memcmp(&tune, &o.tune, sizeof(Tuning)) == 0;
        }
    };
    struct GraphEntry {
        GraphKey key;
        cudaGraphExec_t exec;
        uint64_t last_use;
    };
    std::vector<GraphEntry> graphs;
    std::vector<GraphKey> seen;
    uint64_t use_clock = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ran = false;
    bool profile = false;
    bool direct = false;   // never capture graphs (serving: see batch_direct_launch)
    bool no_spec = false;  // never verify through speculative chain runs (serving)
    bool prof_pending = false;
    PhaseTimer pt;
    std::vector<ProfEntry> prof;
    std::vector<void *> allocs;
};

static int fail(cuspx_ctx *ctx, int code, const std::string &msg) {
    if (ctx) {
        std::lock_guard<std::mutex> lk(ctx->err_mu);
        ctx->err = msg;
    }
    return code;
}

static int cuda_fail(cuspx_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(ctx, CUSPX_ENOMEM, m);
    return fail(ctx, CUSPX_ECUDA, m);
}

#define CK(call, ctx)                                         \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, #call); \
    } while (0)

// The mapping a batch of `count` items of (set, op) runs with: the per-size
// entry whose range holds count, else the set's base mapping.
static const Tuning &effective_tuning(const cuspx_ctx *ctx, int set, int op, size_t count) {
    const int ne = ctx->ntune_for[set][op];
    for (int i = 0; i < ne; i++) {
        const TuneEntry &e = ctx->tune_for[set][op][i];
        if (count >= e.min_count && count <= e.max_count) return e.t;
    }
    return ctx->tune[set];
}

static int load_tuning_file(cuspx_ctx *ctx, const char *path, bool quiet);

extern "C" {

int cuspx_num_sets(void) { return kNumSets; }

int cuspx_set_id(const char *name) {
    if (!name) return CUSPX_EINVAL;
    int id = set_by_name(name);
    return id < 0 ? CUSPX_EINVAL : id;
}

const char *cuspx_set_name(int set) {
    if (set < 0 || set >= kNumSets) return nullptr;
    return kSets[set].name;
}

int cuspx_set_sizes(int set, size_t *pk, size_t *sk, size_t *sig, size_t *seed, int *n) {
    if (set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    SetParams P = make_params(kSets[set]);
    if (pk) *pk = P.pk_bytes;
    if (sk) *sk = P.sk_bytes;
    if (sig) *sig = P.sig_bytes;
    if (seed) *seed = 3 * P.n;
    if (n) *n = P.n;
    return CUSPX_OK;
}

int cuspx_create(int device, cuspx_ctx **out) {
    if (!out) return CUSPX_EINVAL;
    *out = nullptr;
    // Concurrent batches and serving launches use many streams; with the
    // default 8 hardware work queues, streams share queues and a short launch
    // can wait behind a long kernel of another stream.  Ask for 32 (read when
    // the process creates its CUDA context; a caller's own setting is kept).
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    register_all();
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) return CUSPX_ECUDA;
    cuspx_ctx *c = new cuspx_ctx();
    c->device = device;
    // default mappings by set shape (what the autotuner settled on for the
    // reference sets on GB300): one lane per FORS tree for short FORS trees,
    // a lane per XMSS subtree for subtrees of height <= 4, 256-thread leaf
    // blocks where registers allow it (SHA-256 simple)
    for (int i = 0; i < kNumSets; i++) {
        const SetDesc &sd = kSets[i];
        Tuning &t = c->tune[i];
        t.fors_lanes_log2 = sd.a <= 8 ? 0 : std::min(5, sd.a - 6);
        t.tree_mode = sd.h / sd.d <= 4 ? 1 : 0;
        t.leaf_block = (sd.hash == 0 && !sd.robust) ? 256 : 128;
        t.chains_per_warp = sd.hash == 1 ? 256 : 128;
        t.verify_mode = 2;
        // a robust item is several units per F and H: fewer items per warp
        // keep enough warps busy (16384 SHAKE-256f-robust: 2 slots 93.9 ms,
        // 4 slots 98.9 ms; 4096 SHA-256-192f-robust 11.9 / 12.8 ms), except
        // robust SHA-256 at n = 32 (4096 SHA-256-256f-robust 22.8 / 21.1 ms)
        if (sd.robust && !(sd.hash == 0 && sd.n == 32)) t.verify_slots = 2;
        // one item per block up to 128 items: SHA-256-128f 1 item 0.98 ms
        // against 1.18 ms persistent, 128 items 1.00 / 1.20 ms, 256 items
        // 1.44 / 1.22 ms (SHAKE-256f and robust SHA-256-192f cross over
        // between 64 and 256 as well)
        t.verify_item_max = 128;
        // the sorted layered verify from 2048 items; from 1024 for the
        // SHA-256 f sets and robust SHA-256, from 512 for robust SHA-256 at
        // n = 32 and 192f (4096 SHA-256-128f 2.31 ms against 3.65 ms
        // persistent, 1024 items 1.39 / 1.64 ms, 512 items 1.38 / 1.42 ms;
        // SHAKE-256f 1024 items 4.33 / 4.05 ms, 2048 items 6.76 / 8.09 ms;
        // SHA-256-256f-robust 512 items 4.70 / 9.70 ms, SHA-256-128f-robust
        // 512 items 2.92 / 2.76 ms, 1024 items 2.99 / 3.36 ms)
        // speculative chains up to 32 items, 64 for robust SHA-256 (1 item
        // SHA-256-128f 0.54 ms against 0.88 ms one block per item, 32 items
        // 0.78 / 0.87 ms, 64 items 0.95 / 0.88 ms; SHA-256-192f-robust 1 item
        // 1.62 / 3.33 ms, 64 items 2.83 / 3.47 ms; SHAKE-256f 1 item 2.01 /
        // 3.09 ms, 32 items 3.03 / 3.12 ms)
        t.verify_spec_max = (sd.hash == 0 && sd.robust) ? 64 : 32;
        const bool f_set = sd.h / sd.d <= 4;
        if (sd.hash == 0 && sd.robust) t.verify_sorted_min = (sd.n == 32 || (sd.n == 24 && f_set)) ? 512 : 1024;
        else t.verify_sorted_min = (sd.hash == 0 && f_set) ? 1024 : 2048;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        delete c;
        return CUSPX_ECUDA;
    }
    // tuned mappings from the autotuner's file, if there is one for this GPU
    {
        const char *tp = getenv("CUSPX_TUNE_CACHE");
        std::string path;
        if (tp && *tp) path = tp;
        else if (const char *home = getenv("HOME")) path = std::string(home) + "/.cache/cuspx/tune.tsv";
        if (!path.empty()) load_tuning_file(c, path.c_str(), true);
    }
    // the one-shot calls' pinned staging, so that the first call does not
    // pay for the allocation (it grows on demand for larger batches)
    if (cudaMallocHost((void **)&c->stage, (size_t)1 << 20) == cudaSuccess) c->stage_cap = (size_t)1 << 20;
    else c->stage = nullptr;
    cudaGetLastError();
    *out = c;
    return CUSPX_OK;
}

void cuspx_destroy(cuspx_ctx *ctx) {
    if (!ctx) return;
    for (auto &g : ctx->groups) {
        cudaStreamSynchronize(g.origin);
        cudaGraphExecDestroy(g.exec);
        cudaEventDestroy(g.e0);
        cudaEventDestroy(g.e1);
        cudaStreamDestroy(g.origin);
    }
    for (auto &row : ctx->oneshot)
        for (auto *b : row)
            if (b) cuspx_batch_destroy(b);
    if (ctx->stage) cudaFreeHost(ctx->stage);
    delete ctx;
}

// the context's last failure, copied for the calling thread (another thread
// may record a new one meanwhile)
const char *cuspx_error(const cuspx_ctx *ctx) {
    if (!ctx) return "null context";
    static thread_local std::string copy;
    cuspx_ctx *c = const_cast<cuspx_ctx *>(ctx);
    std::lock_guard<std::mutex> lk(c->err_mu);
    copy = c->err;
    return copy.c_str();
}

}  // extern "C"

// base with the fields of `in` applied (cuspx_set_tuning's rules)
static int merge_tuning(cuspx_ctx *ctx, const Tuning &base, const cuspx_tuning *in, Tuning &out) {
    Tuning t = base;
    auto blk = [&](int v, int &dst, const char *what) -> bool {
        if (v <= 0) return true;
        if (v % 32 || v > 1024) {
            fail(ctx, CUSPX_EINVAL, std::string(what) + " must be a multiple of 32 <= 1024");
            return false;
        }
        dst = v;
        return true;
    };
    if (!blk(in->leaf_block, t.leaf_block, "leaf_block") || !blk(in->fors_block, t.fors_block, "fors_block") ||
        !blk(in->verify_block, t.verify_block, "verify_block"))
        return CUSPX_EINVAL;
    if (in->tree_warps > 0) {
        if (in->tree_warps > 32) return fail(ctx, CUSPX_EINVAL, "tree_warps must be <= 32");
        t.tree_warps = in->tree_warps;
    }
    if (in->chains_per_warp > 0) {
        if (in->chains_per_warp < 32 || in->chains_per_warp > 65536)
            return fail(ctx, CUSPX_EINVAL, "chains_per_warp must be in [32, 65536]");
        t.chains_per_warp = in->chains_per_warp;
    }
    if (in->verify_mode >= 0) {
        if (in->verify_mode > 3) return fail(ctx, CUSPX_EINVAL, "verify_mode must be in 0..3");
        t.verify_mode = in->verify_mode;
    }
    if (in->fors_lanes_log2 >= 0) {
        if (in->fors_lanes_log2 > 5) return fail(ctx, CUSPX_EINVAL, "fors_lanes_log2 must be in 0..5");
        t.fors_lanes_log2 = in->fors_lanes_log2;
    }
    if (in->tree_mode >= 0) {
        if (in->tree_mode > 1) return fail(ctx, CUSPX_EINVAL, "tree_mode must be 0 or 1");
        t.tree_mode = in->tree_mode;
    }
    if (in->chain_mode_max >= 0) t.chain_mode_max = in->chain_mode_max;
    if (in->verify_slots > 0) {
        if (in->verify_slots > 8) return fail(ctx, CUSPX_EINVAL, "verify_slots must be in 1..8");
        t.verify_slots = in->verify_slots;
    }
    if (in->verify_item_max >= 0) t.verify_item_max = in->verify_item_max;
    if (in->verify_claim_min > 0) {
        if (in->verify_claim_min > 32) return fail(ctx, CUSPX_EINVAL, "verify_claim_min must be in 1..32");
        t.verify_claim_min = in->verify_claim_min;
    }
    if (in->verify_groups > 0) {
        if (in->verify_groups > VerifyFork::kMaxGroups) return fail(ctx, CUSPX_EINVAL, "verify_groups must be in 1..8");
        t.verify_groups = in->verify_groups;
    }
    if (in->verify_sorted_min >= 0) t.verify_sorted_min = in->verify_sorted_min;
    if (in->verify_spec_max >= 0) {
        if (in->verify_spec_max > kSpecItems) return fail(ctx, CUSPX_EINVAL, "verify_spec_max must be in 0..64");
        t.verify_spec_max = in->verify_spec_max;
    }
    out = t;
    return CUSPX_OK;
}

extern "C" {

int cuspx_set_tuning(cuspx_ctx *ctx, int set, const cuspx_tuning *in) {
    if (!ctx || !in || set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    std::lock_guard<std::mutex> lk(ctx->mu);
    Tuning t;
    if (int rc = merge_tuning(ctx, ctx->tune[set], in, t)) return rc;
    ctx->tune[set] = t;   // batches re-capture their graph when the mapping changed
    return CUSPX_OK;
}

int cuspx_set_tuning_for(cuspx_ctx *ctx, int set, int op, size_t min_count, size_t max_count,
                         const cuspx_tuning *in) {
    if (!ctx || !in || set < 0 || set >= kNumSets || op < 0 || op > 2 || min_count == 0 || max_count < min_count)
        return CUSPX_EINVAL;
    std::lock_guard<std::mutex> lk(ctx->mu);
    Tuning t;
    if (int rc = merge_tuning(ctx, ctx->tune[set], in, t)) return rc;
    TuneEntry *e = ctx->tune_for[set][op];
    int &ne = ctx->ntune_for[set][op];
    for (int i = 0; i < ne; i++) {
        if (e[i].min_count == min_count && e[i].max_count == max_count) {
            e[i].t = t;   // the same range again: replace
            return CUSPX_OK;
        }
        if (min_count <= e[i].max_count && e[i].min_count <= max_count)
            return fail(ctx, CUSPX_EINVAL, "set_tuning_for: range overlaps an existing entry");
    }
    if (ne == kMaxTuneEntries) return fail(ctx, CUSPX_ENOMEM, "set_tuning_for: 16 entries per set and op");
    int i = 0;
    while (i < ne && e[i].min_count < min_count) i++;
    for (int j = ne; j > i; j--) e[j] = e[j - 1];
    e[i] = TuneEntry{min_count, max_count, t};
    ne++;
    return CUSPX_OK;
}

int cuspx_clear_tuning_for(cuspx_ctx *ctx, int set, int op) {
    if (!ctx || set < 0 || set >= kNumSets || op > 2) return CUSPX_EINVAL;
    std::lock_guard<std::mutex> lk(ctx->mu);
    for (int o = 0; o < 3; o++)
        if (op < 0 || o == op) ctx->ntune_for[set][o] = 0;
    return CUSPX_OK;
}

static void to_abi(const Tuning &t, cuspx_tuning *out) {
    out->leaf_block = t.leaf_block;
    out->fors_block = t.fors_block;
    out->verify_block = t.verify_block;
    out->tree_warps = t.tree_warps;
    out->chains_per_warp = t.chains_per_warp;
    out->verify_mode = t.verify_mode;
    out->fors_lanes_log2 = t.fors_lanes_log2;
    out->tree_mode = t.tree_mode;
    out->chain_mode_max = t.chain_mode_max;
    out->verify_slots = t.verify_slots;
    out->verify_item_max = t.verify_item_max;
    out->verify_claim_min = t.verify_claim_min;
    out->verify_groups = t.verify_groups;
    out->verify_sorted_min = t.verify_sorted_min;
    out->verify_spec_max = t.verify_spec_max;
}

int cuspx_get_tuning_for(cuspx_ctx *ctx, int set, int op, size_t count, cuspx_tuning *out) {
    if (!ctx || !out || set < 0 || set >= kNumSets || op < 0 || op > 2) return CUSPX_EINVAL;
    std::lock_guard<std::mutex> lk(ctx->mu);
    to_abi(effective_tuning(ctx, set, op, count), out);
    return CUSPX_OK;
}

int cuspx_load_tuning(cuspx_ctx *ctx, const char *path) {
    if (!ctx || !path) return CUSPX_EINVAL;
    return load_tuning_file(ctx, path, false);
}

int cuspx_device_name(int device, char *buf, size_t len) {
    if (!buf || len == 0) return CUSPX_EINVAL;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        cudaGetLastError();
        return CUSPX_ECUDA;
    }
    snprintf(buf, len, "%s", prop.name);
    return CUSPX_OK;
}

int cuspx_get_tuning(cuspx_ctx *ctx, int set, cuspx_tuning *out) {
    if (!ctx || !out || set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    to_abi(ctx->tune[set], out);
    return CUSPX_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// tuning file (written by cuspx_gb300/autotune.py): one entry per line,
//   <gpu> TAB <set> TAB <sign|verify|keygen> TAB <min_count> TAB <max_count> TAB <ms> TAB <knob>=<v>,...
// Lines of another GPU, unknown sets or knobs, and malformed lines are skipped.
// ---------------------------------------------------------------------------
static int load_tuning_file(cuspx_ctx *ctx, const char *path, bool quiet) {
    FILE *f = fopen(path, "r");
    if (!f) return quiet ? 0 : fail(ctx, CUSPX_EINVAL, std::string("load_tuning: cannot open ") + path);
    char gpu[256] = {0};
    if (cuspx_device_name(ctx->device, gpu, sizeof gpu) != CUSPX_OK) {
        fclose(f);
        return CUSPX_ECUDA;
    }
    int installed = 0;
    char line[2048];
    while (fgets(line, sizeof line, f)) {
        std::vector<std::string> col;
        std::string cur;
        for (const char *p = line; *p && *p != '\n' && *p != '\r'; p++) {
            if (*p == '\t') {
                col.push_back(cur);
                cur.clear();
            } else {
                cur += *p;
            }
        }
        col.push_back(cur);
        if (col.size() != 7 || col[0] != gpu) continue;
        const int set = set_by_name(col[1].c_str());
        const int op = col[2] == "sign" ? CUSPX_OP_SIGN : col[2] == "verify" ? CUSPX_OP_VERIFY
                                                        : col[2] == "keygen" ? CUSPX_OP_KEYGEN : -1;
        const long long lo = atoll(col[3].c_str()), hi = atoll(col[4].c_str());
        if (set < 0 || op < 0 || lo <= 0 || hi < lo) continue;
        cuspx_tuning t;
        t.leaf_block = t.fors_block = t.verify_block = t.tree_warps = t.chains_per_warp = t.verify_slots = 0;
        t.verify_mode = t.fors_lanes_log2 = t.tree_mode = t.chain_mode_max = t.verify_item_max = -1;
        t.verify_claim_min = t.verify_groups = 0;
        t.verify_sorted_min = t.verify_spec_max = -1;
        bool ok = true;
        size_t at = 0;
        const std::string &kv = col[6];
        while (ok && at < kv.size()) {
            size_t end = kv.find(',', at);
            if (end == std::string::npos) end = kv.size();
            const std::string item = kv.substr(at, end - at);
            at = end + 1;
            const size_t eq = item.find('=');
            if (eq == std::string::npos) {
                ok = false;
                break;
            }
            const std::string k = item.substr(0, eq);
            const int v = atoi(item.c_str() + eq + 1);
            if (k == "leaf_block") t.leaf_block = v;
            else if (k == "fors_block") t.fors_block = v;
            else if (k == "verify_block") t.verify_block = v;
            else if (k == "tree_warps") t.tree_warps = v;
            else if (k == "chains_per_warp") t.chains_per_warp = v;
            else if (k == "verify_mode") t.verify_mode = v;
            else if (k == "fors_lanes_log2") t.fors_lanes_log2 = v;
            else if (k == "tree_mode") t.tree_mode = v;
            else if (k == "chain_mode_max") t.chain_mode_max = v;
            else if (k == "verify_slots") t.verify_slots = v;
            else if (k == "verify_item_max") t.verify_item_max = v;
            else if (k == "verify_claim_min") t.verify_claim_min = v;
            else if (k == "verify_groups") t.verify_groups = v;
            else if (k == "verify_sorted_min") t.verify_sorted_min = v;
            else if (k == "verify_spec_max") t.verify_spec_max = v;
            else ok = false;
        }
        if (ok && cuspx_set_tuning_for(ctx, set, op, (size_t)lo, (size_t)hi, &t) == CUSPX_OK) installed++;
    }
    fclose(f);
    return installed;
}

extern "C" {

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
static int balloc(cuspx_batch *b, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return CUSPX_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(b->ctx, e, "cudaMalloc");
    }
    b->allocs.push_back(*p);
    return CUSPX_OK;
}

int cuspx_batch_create(cuspx_ctx *ctx, int op, int set, size_t capacity, size_t msg_capacity, size_t key_capacity,
                       cuspx_batch **out) {
    if (!ctx || !out || set < 0 || set >= kNumSets || op < 0 || op > 2 || capacity == 0 || capacity > (1u << 30))
        return fail(ctx, CUSPX_EINVAL, "batch_create: bad argument");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device), ctx);
    const SetDesc &sd = kSets[set];
    FamilyOps &ops = g_family[sd.hash][sd.n / 8 - 2][sd.robust];
    {
        std::lock_guard<std::mutex> lk(ctx->cfg_mu);
        if (!ctx->configured[sd.hash][sd.n / 8 - 2][sd.robust]) {
            CK(ops.configure(), ctx);
            ctx->configured[sd.hash][sd.n / 8 - 2][sd.robust] = true;
        }
    }
    cuspx_batch *b = new cuspx_batch();
    b->ctx = ctx;
    b->op = op;
    b->set = set;
    b->P = make_params(sd);
    b->cap = capacity;
    b->msg_cap = msg_capacity;
    b->key_cap = key_capacity ? key_capacity : capacity;
    const SetParams &P = b->P;
    const size_t n = P.n, cap = capacity;
    int rc = CUSPX_OK;
    auto A = [&](void **p, size_t bytes) {
        if (rc == CUSPX_OK) rc = balloc(b, p, bytes);
    };
    if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return fail(ctx, CUSPX_ECUDA, "cudaStreamCreate");
    }
    cudaEventCreate(&b->e0);
    cudaEventCreate(&b->e1);
    for (auto &e : b->pt.ev) cudaEventCreate(&e);
    if (op == CUSPX_OP_VERIFY) {
        VerifyFork &vf = b->vfork;
        bool ok = cudaEventCreateWithFlags(&vf.fork, cudaEventDisableTiming) == cudaSuccess;
        for (int g = 0; ok && g + 1 < VerifyFork::kMaxGroups; g++) {
            ok = cudaStreamCreateWithFlags(&vf.side[g], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&vf.join[g], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&vf.chain[g], cudaEventDisableTiming) == cudaSuccess;
            if (ok) vf.sides = g + 1;
        }
        if (!ok) {
            cuspx_batch_destroy(b);
            return fail(ctx, CUSPX_ECUDA, "verify side streams");
        }
    }
    if (op == CUSPX_OP_SIGN) {
        if (cudaStreamCreateWithFlags(&b->fork.side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->fork.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->fork.join, cudaEventDisableTiming) != cudaSuccess) {
            cuspx_batch_destroy(b);
            return fail(ctx, CUSPX_ECUDA, "side stream");
        }
    }
    const size_t keyrow_bytes = op == CUSPX_OP_VERIFY ? 2 * n : 4 * n;
    A((void **)&b->keys, b->key_cap * keyrow_bytes);
    A((void **)&b->status, cap * sizeof(int32_t));
    if (op == CUSPX_OP_KEYGEN) {
        A((void **)&b->out, cap * 2 * n);
        A((void **)&b->leaves, cap * ((size_t)1 << P.hp) * n);
        A((void **)&b->roots, cap * n);
        // chain-parallel scratch
        b->ends_cap = (uint32_t)std::min<size_t>(cap, kKeygenChainItems);
        A((void **)&b->ends, (size_t)b->ends_cap * ((size_t)1 << P.hp) * P.len * n);
    } else {
        A((void **)&b->keyrow, cap * sizeof(uint32_t));
        A((void **)&b->msg, msg_capacity + 64);
        A((void **)&b->off, cap * sizeof(uint64_t));
        A((void **)&b->len, cap * sizeof(uint64_t));
        A((void **)&b->work, cap * sizeof(SignWork));
        A((void **)&b->fors_roots, cap * P.k * n);
        if (op == CUSPX_OP_SIGN) {
            A((void **)&b->aux, cap * n);
            A((void **)&b->out, cap * P.sig_bytes);
            A((void **)&b->leaves, cap * P.d * ((size_t)1 << P.hp) * n);
            A((void **)&b->roots, cap * P.d * n);
            A((void **)&b->chains, cap * P.d * P.len * 16 * n);
            // chain-parallel scratch for small batches
            b->ends_cap = (uint32_t)std::min<size_t>(cap, kChainModeItems);
            A((void **)&b->ends, (size_t)b->ends_cap * P.d * ((size_t)1 << P.hp) * P.len * n);
        } else {
            A((void **)&b->aux, cap * P.sig_bytes);
            A((void **)&b->siglen, cap * sizeof(uint64_t));
            A((void **)&b->wpk, cap * P.len * n);
            A((void **)&b->cur_root, cap * n);
            A((void **)&b->ctr, 16);
            b->vlists.stride = cap * P.len;
            A((void **)&b->vlists.tasks, 16 * b->vlists.stride * sizeof(uint32_t));
            A((void **)&b->vlists.cnt, (size_t)VerifyFork::kMaxGroups * P.d * 16 * sizeof(uint32_t));
        }
    }
    if (rc != CUSPX_OK) {
        cuspx_batch_destroy(b);   // records nothing: the allocation failure's message stays
        return rc;
    }
    *out = b;
    return CUSPX_OK;
}

void cuspx_batch_destroy(cuspx_batch *b) {
    if (!b) return;
    if (b->s) cudaStreamSynchronize(b->s);
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.exec);
    for (void *p : b->allocs) cudaFree(p);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    for (auto &e : b->pt.ev)
        if (e) cudaEventDestroy(e);
    if (b->fork.side) {
        cudaStreamSynchronize(b->fork.side);
        cudaStreamDestroy(b->fork.side);
    }
    if (b->fork.fork) cudaEventDestroy(b->fork.fork);
    if (b->fork.join) cudaEventDestroy(b->fork.join);
    for (int g = 0; g + 1 < VerifyFork::kMaxGroups; g++) {
        if (b->vfork.side[g]) {
            cudaStreamSynchronize(b->vfork.side[g]);
            cudaStreamDestroy(b->vfork.side[g]);
        }
        if (b->vfork.join[g]) cudaEventDestroy(b->vfork.join[g]);
        if (b->vfork.chain[g]) cudaEventDestroy(b->vfork.chain[g]);
    }
    if (b->vfork.fork) cudaEventDestroy(b->vfork.fork);
    if (b->s && b->own_stream) cudaStreamDestroy(b->s);
    delete b;
}

int cuspx_batch_upload(cuspx_batch *b, size_t count, const uint8_t *keys, size_t nkeys, const uint32_t *key_index,
                       const uint8_t *msgs, size_t msg_bytes, const uint64_t *msg_off, const uint64_t *msg_len,
                       const uint8_t *aux, const uint64_t *siglens) {
    if (!b) return CUSPX_EINVAL;
    cuspx_ctx *ctx = b->ctx;
    const SetParams &P = b->P;
    const size_t n = P.n;
    if (count > b->cap) return fail(ctx, CUSPX_EINVAL, "upload: count exceeds batch capacity");
    const bool bound = b->bound_keys != nullptr && b->op != CUSPX_OP_KEYGEN;
    if (count && !keys && !bound) return fail(ctx, CUSPX_EINVAL, "upload: keys is null");
    CK(cudaSetDevice(ctx->device), ctx);
    if (b->op == CUSPX_OP_KEYGEN) {
        // seeds (count x 3n) into the first 3n bytes of each sk row
        if (count) CK(cudaMemcpy2DAsync(b->keys, 4 * n, keys, 3 * n, 3 * n, count, cudaMemcpyHostToDevice, b->s), ctx);
        b->count = count;
        return CUSPX_OK;
    }
    if (bound && !keys) nkeys = b->bound_nkeys;
    if (nkeys == 0) nkeys = count;
    if (!bound && nkeys > b->key_cap) return fail(ctx, CUSPX_EINVAL, "upload: more keys than key capacity");
    if (key_index) {
        for (size_t i = 0; i < count; i++)
            if (key_index[i] >= nkeys) return fail(ctx, CUSPX_EINVAL, "upload: key_index out of range");
    } else if (nkeys < count) {
        return fail(ctx, CUSPX_EINVAL, "upload: fewer keys than items and no key_index");
    }
    if (count && (!msg_off || !msg_len)) return fail(ctx, CUSPX_EINVAL, "upload: message offsets/lengths are null");
    for (size_t i = 0; i < count; i++) {
        if (msg_off[i] % 16) return fail(ctx, CUSPX_EINVAL, "upload: message offsets must be multiples of 16");
        if (msg_off[i] + msg_len[i] > msg_bytes || msg_off[i] + msg_len[i] < msg_off[i])
            return fail(ctx, CUSPX_EINVAL, "upload: message outside the message buffer");
    }
    if (msg_bytes > b->msg_cap) return fail(ctx, CUSPX_EINVAL, "upload: messages exceed message capacity");
    const size_t krow = b->op == CUSPX_OP_VERIFY ? 2 * n : 4 * n;
    if (keys && bound) return fail(ctx, CUSPX_EINVAL, "upload: batch is bound to a resident key table");
    if (nkeys && keys) CK(cudaMemcpyAsync(b->keys, keys, nkeys * krow, cudaMemcpyHostToDevice, b->s), ctx);
    if (key_index && count) CK(cudaMemcpyAsync(b->keyrow, key_index, count * 4, cudaMemcpyHostToDevice, b->s), ctx);
    if (msg_bytes) CK(cudaMemcpyAsync(b->msg, msgs, msg_bytes, cudaMemcpyHostToDevice, b->s), ctx);
    if (count) {
        CK(cudaMemcpyAsync(b->off, msg_off, count * 8, cudaMemcpyHostToDevice, b->s), ctx);
        CK(cudaMemcpyAsync(b->len, msg_len, count * 8, cudaMemcpyHostToDevice, b->s), ctx);
    }
    b->long_msgs = false;
    for (size_t i = 0; i < count && !b->long_msgs; i++) b->long_msgs = msg_len[i] >= kPairMsgBytes;
    b->use_keyrow = key_index != nullptr;
    if (b->op == CUSPX_OP_SIGN) {
        b->use_aux = aux != nullptr;
        if (aux && count) CK(cudaMemcpyAsync(b->aux, aux, count * n, cudaMemcpyHostToDevice, b->s), ctx);
    } else {
        if (count && !aux) return fail(ctx, CUSPX_EINVAL, "upload: signatures are null");
        if (count) CK(cudaMemcpyAsync(b->aux, aux, count * P.sig_bytes, cudaMemcpyHostToDevice, b->s), ctx);
        b->use_siglen = siglens != nullptr;
        if (siglens && count) CK(cudaMemcpyAsync(b->siglen, siglens, count * 8, cudaMemcpyHostToDevice, b->s), ctx);
    }
    b->count = count;
    return CUSPX_OK;
}

// FORS on a side stream beside the hypertree (0: one stream, for A/B runs)
#ifndef CUSPX_SIGN_FORK
#define CUSPX_SIGN_FORK 1
#endif

static void launch_seq(cuspx_batch *b, PhaseTimer *pt) {
    const FamilyOps &ops = family_of(b->set);
    const Tuning &tu = effective_tuning(b->ctx, b->set, b->op, b->count);
    const SetParams &P = b->P;
    const uint32_t cnt = (uint32_t)b->count;
    if (b->op == CUSPX_OP_SIGN) {
        SignArgs A;
        A.count = cnt;
        A.sk = KeyRef{b->bound_keys ? b->bound_keys : b->keys, b->use_keyrow ? b->keyrow : nullptr,
                      (uint32_t)P.sk_bytes};
        A.msg = MsgRef{b->msg, b->off, b->len};
        A.optrand = b->use_aux ? b->aux : nullptr;
        A.sig = b->out;
        A.work = b->work;
        A.fors_roots = b->fors_roots;
        A.leaves = b->leaves;
        A.roots = b->roots;
        A.chains = b->chains;
        A.status = b->status;
        A.ends = b->ends;
        A.ends_cap = b->ends_cap;
        ops.sign(P, A, tu, b->s, pt, b->long_msgs ? kPairMsgBytes : 0,
                 (CUSPX_SIGN_FORK && b->fork.side) ? &b->fork : nullptr);
    } else if (b->op == CUSPX_OP_VERIFY) {
        VerifyArgs A;
        A.count = cnt;
        A.pk = KeyRef{b->bound_keys ? b->bound_keys : b->keys, b->use_keyrow ? b->keyrow : nullptr,
                      (uint32_t)P.pk_bytes};
        A.msg = MsgRef{b->msg, b->off, b->len};
        A.sig = b->aux;
        A.sig_stride = P.sig_bytes;
        A.siglen = b->use_siglen ? b->siglen : nullptr;
        A.work = b->work;
        A.fors_roots = b->fors_roots;
        A.verdict = b->status;
        A.wpk = b->wpk;
        A.cur_root = b->cur_root;
        A.ctr = b->ctr;
        ops.verify(P, A, tu, b->s, pt, b->long_msgs ? kPairMsgBytes : 0, &b->vlists, &b->vfork);
    } else {
        KeygenArgs K{cnt, b->keys, b->out, b->leaves, b->roots, b->ends, b->ends_cap};
        ops.keygen(P, K, tu, b->s, pt);
    }
}

static void collect_profile(cuspx_batch *b) {
    if (!b->prof_pending) return;
    b->prof_pending = false;
    for (int i = 0; i < b->pt.n; i++) {
        float ms = 0;
        cudaEventElapsedTime(&ms, b->pt.ev[i], b->pt.ev[i + 1]);
        auto it = std::find_if(b->prof.begin(), b->prof.end(),
                               [&](const ProfEntry &e) { return !strcmp(e.name, b->pt.names[i]); });
        if (it == b->prof.end()) b->prof.push_back(ProfEntry{b->pt.names[i], ms, 1});
        else {
            it->ms += ms;
            it->launches++;
        }
    }
}

// The speculative chain table of a verify batch, allocated the first time a
// batch runs at a size the speculative path takes (outside any capture: the
// first run of a shape is a direct launch, and group_run calls this before
// it captures).  If the allocation fails the batch verifies without it.
static void spec_scratch(cuspx_batch *b) {
    if (b->op != CUSPX_OP_VERIFY || b->vlists.cand || b->no_spec) return;
    const Tuning &tu = effective_tuning(b->ctx, b->set, b->op, b->count);
    if (tu.verify_spec_max <= 0 || b->count > (size_t)tu.verify_spec_max) return;
    const SetParams &P = b->P;
    const size_t items = std::min<size_t>(b->cap, kSpecItems);
    void *p = nullptr;
    if (cudaMalloc(&p, items * P.d * P.len * 16 * P.n) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    b->allocs.push_back(p);
    b->vlists.cand = (uint8_t *)p;
    b->vlists.cand_items = (uint32_t)items;
}

int cuspx_batch_run(cuspx_batch *b) {
    if (!b) return CUSPX_EINVAL;
    cuspx_ctx *ctx = b->ctx;
    CK(cudaSetDevice(ctx->device), ctx);
    if (b->count == 0) return CUSPX_OK;
    spec_scratch(b);
    if (b->profile) {
        collect_profile(b);
        b->pt.n = 0;
        CK(cudaEventRecord(b->pt.ev[0], b->s), ctx);
        CK(cudaEventRecord(b->e0, b->s), ctx);
        launch_seq(b, &b->pt);
        CK(cudaGetLastError(), ctx);
        CK(cudaEventRecord(b->e1, b->s), ctx);
        b->prof_pending = true;
        b->ran = true;
        return CUSPX_OK;
    }
    if (b->direct) {
        CK(cudaEventRecord(b->e0, b->s), ctx);
        launch_seq(b, nullptr);
        CK(cudaGetLastError(), ctx);
        CK(cudaEventRecord(b->e1, b->s), ctx);
        b->ran = true;
        return CUSPX_OK;
    }
    const Tuning &tu = effective_tuning(ctx, b->set, b->op, b->count);
    cuspx_batch::GraphKey key{b->count, b->use_keyrow, b->use_aux, b->use_siglen, b->long_msgs, b->bound_keys, tu};
    b->use_clock++;
    cuspx_batch::GraphEntry *hit = nullptr;
    for (auto &g : b->graphs)
        if (g.key == key) hit = &g;
    if (!hit) {
        const bool second = std::find(b->seen.begin(), b->seen.end(), key) != b->seen.end();
        if (!second) {
            // first use of this shape: launch directly, remember it
            if (b->seen.size() >= 64) b->seen.erase(b->seen.begin());
            b->seen.push_back(key);
            CK(cudaEventRecord(b->e0, b->s), ctx);
            launch_seq(b, nullptr);
            CK(cudaGetLastError(), ctx);
            CK(cudaEventRecord(b->e1, b->s), ctx);
            b->ran = true;
            return CUSPX_OK;
        }
        cudaGraph_t g;
        cudaGraphExec_t exec = nullptr;
        CK(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal), ctx);
        launch_seq(b, nullptr);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(b->s, &g);
        if (le != cudaSuccess) return cuda_fail(ctx, le, "launch during capture");
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return cuda_fail(ctx, ie, "cudaGraphInstantiate");
        if (b->graphs.size() >= 8) {
            auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                        [](const cuspx_batch::GraphEntry &x, const cuspx_batch::GraphEntry &y) {
                                            return x.last_use < y.last_use;
                                        });
            cudaGraphExecDestroy(lru->exec);
            b->graphs.erase(lru);
        }
        b->graphs.push_back(cuspx_batch::GraphEntry{key, exec, 0});
        hit = &b->graphs.back();
    }
    hit->last_use = b->use_clock;
    CK(cudaEventRecord(b->e0, b->s), ctx);
    CK(cudaGraphLaunch(hit->exec, b->s), ctx);
    CK(cudaEventRecord(b->e1, b->s), ctx);
    b->ran = true;
    return CUSPX_OK;
}

int cuspx_batch_sync(cuspx_batch *b) {
    if (!b) return CUSPX_EINVAL;
    CK(cudaStreamSynchronize(b->s), b->ctx);
    collect_profile(b);
    return CUSPX_OK;
}

int cuspx_batch_download_async(cuspx_batch *b, uint8_t *out, uint8_t *out2, int32_t *status) {
    if (!b) return CUSPX_EINVAL;
    cuspx_ctx *ctx = b->ctx;
    CK(cudaSetDevice(ctx->device), ctx);
    const SetParams &P = b->P;
    const size_t cnt = b->count;
    if (!cnt) return CUSPX_OK;
    if (b->op == CUSPX_OP_SIGN) {
        if (out) CK(cudaMemcpyAsync(out, b->out, cnt * P.sig_bytes, cudaMemcpyDeviceToHost, b->s), ctx);
    } else if (b->op == CUSPX_OP_KEYGEN) {
        if (out) CK(cudaMemcpyAsync(out, b->keys, cnt * P.sk_bytes, cudaMemcpyDeviceToHost, b->s), ctx);
        if (out2) CK(cudaMemcpyAsync(out2, b->out, cnt * P.pk_bytes, cudaMemcpyDeviceToHost, b->s), ctx);
    }
    if (status && b->op != CUSPX_OP_KEYGEN)
        CK(cudaMemcpyAsync(status, b->status, cnt * 4, cudaMemcpyDeviceToHost, b->s), ctx);
    return CUSPX_OK;
}

int cuspx_batch_download(cuspx_batch *b, uint8_t *out, uint8_t *out2, int32_t *status) {
    if (!b) return CUSPX_EINVAL;
    int rc = cuspx_batch_download_async(b, out, out2, status);
    if (rc) return rc;
    return cuspx_batch_sync(b);
}

int cuspx_batch_last_ms(cuspx_batch *b, float *ms) {
    if (!b || !ms || !b->ran) return CUSPX_EINVAL;
    CK(cudaEventSynchronize(b->e1), b->ctx);
    CK(cudaEventElapsedTime(ms, b->e0, b->e1), b->ctx);
    return CUSPX_OK;
}

void *cuspx_batch_stream(cuspx_batch *b) { return b ? (void *)b->s : nullptr; }

}  // extern "C"

namespace cuspx {
// Library-internal: launch this batch's kernels directly, never as a
// captured graph.  Serving sees a different item count on almost every
// launch, so it would capture and instantiate graphs while other launches
// run; instantiation can wait for work already on the GPU (tens of ms behind
// a long-message kernel) and holds the driver meanwhile, stalling every
// thread's CUDA calls.  A direct launch of the 4-8 kernels costs tens of us.
void batch_direct_launch(cuspx_batch *b, bool on) {
    if (!b) return;
    b->direct = on;
    // Serving launches stay on one stream: with a second stream per sign
    // slot the <= 1 KiB sign p99 of a mixed 16 B..1 MiB request stream rose
    // from 2.5 to 17 ms (more streams than hardware queues, so short
    // launches queue behind long ones).
    if (on && b->fork.side) {
        cudaStreamSynchronize(b->fork.side);
        cudaStreamDestroy(b->fork.side);
        cudaEventDestroy(b->fork.fork);
        cudaEventDestroy(b->fork.join);
        b->fork = StreamFork{};
    }
    // Likewise a verify batch's side streams (the sorted verify's item
    // groups then share the launch stream).  And no speculative chain runs:
    // they cost ~15 times a verify's chain work, a latency trade for an idle
    // GPU, and under a served load that work queues every other request
    // (a three-set stream at 20k req/s: sign p99 6.6 -> 138 ms).
    if (on) {
        b->no_spec = true;
        for (int g = 0; g + 1 < VerifyFork::kMaxGroups; g++) {
            if (b->vfork.side[g]) {
                cudaStreamSynchronize(b->vfork.side[g]);
                cudaStreamDestroy(b->vfork.side[g]);
            }
            if (b->vfork.join[g]) cudaEventDestroy(b->vfork.join[g]);
            if (b->vfork.chain[g]) cudaEventDestroy(b->vfork.chain[g]);
        }
        if (b->vfork.fork) cudaEventDestroy(b->vfork.fork);
        b->vfork = VerifyFork{};
    }
}

// Library-internal: launch an idle batch that already runs on a caller's
// stream (batch_share_stream) on another of the caller's streams from now
// on.  Nothing is waited for: the caller knows the batch's work is done.
void batch_use_stream(cuspx_batch *b, cudaStream_t s) {
    if (b && s && !b->own_stream) b->s = s;
}

// Library-internal: run an idle batch on a stream owned by the caller (which
// keeps it alive while the batch exists and destroys it afterwards); the
// batch's own stream and captured graphs are dropped.  Several batches may
// share one stream: their launches then run in submission order.
int batch_share_stream(cuspx_batch *b, cudaStream_t s) {
    if (!b || !s) return CUSPX_EINVAL;
    CK(cudaStreamSynchronize(b->s), b->ctx);
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.exec);
    b->graphs.clear();
    if (b->own_stream) cudaStreamDestroy(b->s);
    b->s = s;
    b->own_stream = false;
    return CUSPX_OK;
}
}  // namespace cuspx

extern "C" {

int cuspx_batch_bind_keys(cuspx_batch *b, const void *d_keys, size_t nkeys) {
    if (!b || b->op == CUSPX_OP_KEYGEN) return CUSPX_EINVAL;
    b->bound_keys = (const uint8_t *)d_keys;
    b->bound_nkeys = d_keys ? nkeys : 0;
    return CUSPX_OK;
}

int cuspx_batch_device_ptrs(cuspx_batch *b, void **keys, void **msgs, void **msg_off, void **msg_len, void **aux,
                            void **out, void **status) {
    if (!b) return CUSPX_EINVAL;
    if (keys) *keys = b->keys;
    if (msgs) *msgs = b->msg;
    if (msg_off) *msg_off = b->off;
    if (msg_len) *msg_len = b->len;
    if (aux) *aux = b->aux;
    if (out) *out = b->out;
    if (status) *status = b->status;
    return CUSPX_OK;
}

int cuspx_batch_profile(cuspx_batch *b, int enable) {
    if (!b) return CUSPX_EINVAL;
    if (b->profile && !enable) cuspx_batch_sync(b);
    b->profile = enable != 0;
    if (enable) b->prof.clear();
    return CUSPX_OK;
}

int cuspx_batch_kernel_ms(cuspx_batch *b, int idx, const char **name, double *ms, long *launches) {
    if (!b) return CUSPX_EINVAL;
    cuspx_batch_sync(b);
    if (idx < 0) return (int)b->prof.size();
    if (idx >= (int)b->prof.size()) return CUSPX_EINVAL;
    if (name) *name = b->prof[idx].name;
    if (ms) *ms = b->prof[idx].ms;
    if (launches) *launches = b->prof[idx].launches;
    return CUSPX_OK;
}

// ---------------------------------------------------------------------------
// one-shot host-buffer calls
// ---------------------------------------------------------------------------
static int oneshot_batch(cuspx_ctx *ctx, int op, int set, size_t count, size_t msg_bytes, cuspx_batch **out) {
    cuspx_batch *&b = ctx->oneshot[op][set];
    if (b && (b->cap < count || b->msg_cap < msg_bytes)) {
        cuspx_batch_destroy(b);
        b = nullptr;
    }
    if (!b) {
        size_t cap = std::max<size_t>(count, 1);
        size_t mcap = std::max<size_t>(msg_bytes, 4096);
        int rc = cuspx_batch_create(ctx, op, set, cap, mcap, cap, &b);
        if (rc) {
            b = nullptr;
            return rc;
        }
    }
    *out = b;
    return CUSPX_OK;
}

static size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// Pinned host staging for the one-shot calls (under ctx->mu): their inputs
// are packed here and their outputs land here, so every copy is a direct
// DMA rather than a pass through the driver's pageable bounce buffer (a
// plain one-signature call makes six small copies).  Grown on demand and
// kept for the context's life.
struct Staging {
    uint8_t *base = nullptr;
    size_t used = 0;
    void *take(size_t bytes) {
        void *p = base + used;
        used += al16(bytes);
        return p;
    }
};
static int oneshot_stage(cuspx_ctx *ctx, size_t bytes, Staging &st) {
    if (ctx->stage_cap < bytes) {
        if (ctx->stage) cudaFreeHost(ctx->stage);
        ctx->stage = nullptr;
        ctx->stage_cap = 0;
        const size_t cap = std::max<size_t>(bytes, (size_t)1 << 20);
        if (cudaMallocHost((void **)&ctx->stage, cap) != cudaSuccess) {
            ctx->stage = nullptr;
            cudaGetLastError();
            return fail(ctx, CUSPX_ECUDA, "cudaMallocHost: one-shot staging");
        }
        ctx->stage_cap = cap;
    }
    st.base = ctx->stage;
    st.used = 0;
    return CUSPX_OK;
}
// bytes of the messages packed at 16-byte aligned offsets
static size_t packed_bytes(size_t count, const uint64_t *len) {
    size_t total = 0;
    for (size_t i = 0; i < count; i++) total += al16(len[i]);
    return total;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// One-shot calls from concurrent threads share launches.  Each call becomes
// a job on the context's queue; a caller that finds no launch running takes
// the oldest job and every other queued job of the same operation and set
// (up to kCombineItems items and kCombineBytes of messages), packs them
// into one batch, launches it, and hands every job its slice of the results.
// Callers arriving meanwhile queue for the next launch, so N threads calling
// crypto_sign_signature at once share launches instead of running one
// launch each in turn.  A lone caller sees no difference.
// ---------------------------------------------------------------------------
namespace {
constexpr size_t kCombineItems = 4096;
constexpr size_t kCombineBytes = (size_t)256 << 20;
}  // namespace

struct OneshotJob {
    int op = 0, set = 0;
    size_t count = 0;
    const uint8_t *keys = nullptr;   // seeds (keygen), sk rows (sign), pk rows (verify)
    const uint8_t *msgs = nullptr;
    const uint64_t *off = nullptr, *len = nullptr;
    const uint8_t *aux = nullptr;    // sign: optrand (may be null); verify: signature rows
    const uint64_t *siglens = nullptr;
    uint8_t *out = nullptr;          // sign: signatures; keygen: pk rows
    uint8_t *out2 = nullptr;         // keygen: sk rows
    int32_t *status = nullptr;       // sign: statuses (may be null); verify: verdicts
    size_t msg_bytes = 0;            // its messages packed at 16-byte offsets
    int rc = CUSPX_OK;
    bool done = false;
};

// Run jobs of one (op, set) as one batch; under ctx->mu.
static int oneshot_run(cuspx_ctx *ctx, int op, int set, const std::vector<OneshotJob *> &jobs) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    size_t count = 0, total = 0;
    bool any_opt = false;
    for (const OneshotJob *j : jobs) {
        count += j->count;
        total += j->msg_bytes;
        any_opt |= j->aux != nullptr;
    }
    cuspx_batch *b;
    int rc = oneshot_batch(ctx, op, set, count, total, &b);
    if (rc) return rc;
    const SetParams &P = b->P;
    const size_t n = P.n;
    Staging st;
    if (op == CUSPX_OP_KEYGEN) {
        const size_t seed_b = count * 3 * n, sk_b = count * P.sk_bytes, pk_b = count * P.pk_bytes;
        if ((rc = oneshot_stage(ctx, al16(seed_b) + al16(sk_b) + al16(pk_b), st))) return rc;
        uint8_t *h_seed = (uint8_t *)st.take(seed_b);
        uint8_t *h_sk = (uint8_t *)st.take(sk_b);
        uint8_t *h_pk = (uint8_t *)st.take(pk_b);
        size_t at = 0;
        for (const OneshotJob *j : jobs) {
            memcpy(h_seed + at * 3 * n, j->keys, j->count * 3 * n);
            at += j->count;
        }
        if ((rc = cuspx_batch_upload(b, count, h_seed, count, nullptr, nullptr, 0, nullptr, nullptr, nullptr,
                                     nullptr)))
            return rc;
        if ((rc = cuspx_batch_run(b))) return rc;
        if ((rc = cuspx_batch_download(b, h_sk, h_pk, nullptr))) return rc;
        at = 0;
        for (const OneshotJob *j : jobs) {
            memcpy(j->out2, h_sk + at * P.sk_bytes, j->count * P.sk_bytes);
            memcpy(j->out, h_pk + at * P.pk_bytes, j->count * P.pk_bytes);
            at += j->count;
        }
        return CUSPX_OK;
    }
    const bool sign = op == CUSPX_OP_SIGN;
    const size_t key_b = count * (sign ? P.sk_bytes : P.pk_bytes);
    const size_t opt_b = sign && any_opt ? count * n : 0;
    const size_t sig_b = count * P.sig_bytes;
    const size_t sl_b = sign ? 0 : count * 8;
    if ((rc = oneshot_stage(ctx, al16(key_b) + 2 * al16(count * 8) + al16(opt_b) + al16(sl_b) + al16(total + 16) +
                                     al16(sig_b) + al16(count * 4), st)))
        return rc;
    uint8_t *h_key = (uint8_t *)st.take(key_b);
    uint64_t *h_off = (uint64_t *)st.take(count * 8);
    uint64_t *h_len = (uint64_t *)st.take(count * 8);
    uint8_t *h_opt = opt_b ? (uint8_t *)st.take(opt_b) : nullptr;
    uint64_t *h_sl = sl_b ? (uint64_t *)st.take(sl_b) : nullptr;
    uint8_t *h_msg = (uint8_t *)st.take(total + 16);
    uint8_t *h_sig = (uint8_t *)st.take(sig_b);
    int32_t *h_st = (int32_t *)st.take(count * 4);
    memset(h_msg, 0, total + 16);
    size_t at = 0, o = 0;
    const size_t krow = sign ? P.sk_bytes : P.pk_bytes;
    for (const OneshotJob *j : jobs) {
        memcpy(h_key + at * krow, j->keys, j->count * krow);
        for (size_t i = 0; i < j->count; i++) {
            h_off[at + i] = o;
            h_len[at + i] = j->len[i];
            if (j->len[i]) memcpy(h_msg + o, j->msgs + j->off[i], j->len[i]);
            o += al16(j->len[i]);
        }
        if (h_opt) {
            // a job without optrand gets the reference's fixed 0xAD bytes (sign.cu:1950-1954)
            if (j->aux) memcpy(h_opt + at * n, j->aux, j->count * n);
            else memset(h_opt + at * n, 0xad, j->count * n);
        }
        if (!sign) {
            memcpy(h_sig + at * P.sig_bytes, j->aux, j->count * P.sig_bytes);
            for (size_t i = 0; i < j->count; i++) h_sl[at + i] = j->siglens ? j->siglens[i] : P.sig_bytes;
        }
        at += j->count;
    }
    if ((rc = cuspx_batch_upload(b, count, h_key, count, nullptr, h_msg, total, h_off, h_len,
                                 sign ? h_opt : h_sig, h_sl)))
        return rc;
    if ((rc = cuspx_batch_run(b))) return rc;
    if ((rc = cuspx_batch_download(b, sign ? h_sig : nullptr, nullptr, h_st))) return rc;
    at = 0;
    for (const OneshotJob *j : jobs) {
        if (sign) memcpy(j->out, h_sig + at * P.sig_bytes, j->count * P.sig_bytes);
        if (j->status) memcpy(j->status, h_st + at, j->count * 4);
        at += j->count;
    }
    return CUSPX_OK;
}

// Queue a job and return when it has run (see above).
static int oneshot_submit(cuspx_ctx *ctx, OneshotJob &job) {
    std::unique_lock<std::mutex> lk(ctx->comb_mu);
    ctx->comb_q.push_back(&job);
    while (!job.done) {
        if (ctx->comb_busy) {
            ctx->comb_cv.wait(lk);
            continue;
        }
        ctx->comb_busy = true;
        std::vector<OneshotJob *> take;
        const int op = ctx->comb_q.front()->op, set = ctx->comb_q.front()->set;
        size_t items = 0, bytes = 0;
        for (auto it = ctx->comb_q.begin(); it != ctx->comb_q.end();) {
            OneshotJob *q = *it;
            const bool fits = take.empty() || (items + q->count <= kCombineItems && bytes + q->msg_bytes <= kCombineBytes);
            if (q->op == op && q->set == set && fits) {
                take.push_back(q);
                items += q->count;
                bytes += q->msg_bytes;
                it = ctx->comb_q.erase(it);
            } else {
                ++it;
            }
        }
        lk.unlock();
        const int rc = oneshot_run(ctx, op, set, take);
        lk.lock();
        for (OneshotJob *q : take) {
            q->rc = rc;
            q->done = true;   // its owner may return (and free it) once the lock is released
        }
        ctx->comb_busy = false;
        ctx->comb_cv.notify_all();
    }
    return job.rc;
}

extern "C" {

int cuspx_keypair_batch(cuspx_ctx *ctx, int set, size_t count, const uint8_t *seeds, uint8_t *pks, uint8_t *sks) {
    if (!ctx || set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    if (count == 0) return CUSPX_OK;
    if (!seeds || !pks || !sks) return fail(ctx, CUSPX_EINVAL, "keypair_batch: null buffer");
    OneshotJob j;
    j.op = CUSPX_OP_KEYGEN;
    j.set = set;
    j.count = count;
    j.keys = seeds;
    j.out = pks;
    j.out2 = sks;
    return oneshot_submit(ctx, j);
}

int cuspx_sign_batch(cuspx_ctx *ctx, int set, size_t count, const uint8_t *sks, const uint8_t *msgs,
                     const uint64_t *msg_off, const uint64_t *msg_len, const uint8_t *optrand, uint8_t *sigs,
                     int32_t *status) {
    if (!ctx || set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    if (count == 0) return CUSPX_OK;
    if (!sks || !msg_off || !msg_len || !sigs) return fail(ctx, CUSPX_EINVAL, "sign_batch: null buffer");
    const size_t total = packed_bytes(count, msg_len);
    if (!msgs && total) return fail(ctx, CUSPX_EINVAL, "sign_batch: msgs is null but a message is not empty");
    OneshotJob j;
    j.op = CUSPX_OP_SIGN;
    j.set = set;
    j.count = count;
    j.keys = sks;
    j.msgs = msgs;
    j.off = msg_off;
    j.len = msg_len;
    j.aux = optrand;
    j.out = sigs;
    j.status = status;
    j.msg_bytes = total;
    return oneshot_submit(ctx, j);
}

int cuspx_verify_batch(cuspx_ctx *ctx, int set, size_t count, const uint8_t *pks, const uint8_t *msgs,
                       const uint64_t *msg_off, const uint64_t *msg_len, const uint8_t *sigs,
                       const uint64_t *siglens, int32_t *verdicts) {
    if (!ctx || set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    if (count == 0) return CUSPX_OK;
    if (!pks || !msg_off || !msg_len || !sigs || !verdicts) return fail(ctx, CUSPX_EINVAL, "verify_batch: null buffer");
    const size_t total = packed_bytes(count, msg_len);
    if (!msgs && total) return fail(ctx, CUSPX_EINVAL, "verify_batch: msgs is null but a message is not empty");
    OneshotJob j;
    j.op = CUSPX_OP_VERIFY;
    j.set = set;
    j.count = count;
    j.keys = pks;
    j.msgs = msgs;
    j.off = msg_off;
    j.len = msg_len;
    j.aux = sigs;
    j.siglens = siglens;
    j.status = verdicts;
    j.msg_bytes = total;
    return oneshot_submit(ctx, j);
}

// ---------------------------------------------------------------------------
// mixed parameter sets in one graph launch
// ---------------------------------------------------------------------------
int cuspx_group_run(cuspx_ctx *ctx, cuspx_batch *const *batches, int nb, float *ms) {
    if (!ctx || !batches || nb <= 0 || nb > 64) return CUSPX_EINVAL;
    for (int i = 0; i < nb; i++)
        if (!batches[i] || batches[i]->ctx != ctx || batches[i]->profile)
            return fail(ctx, CUSPX_EINVAL, "group_run: batch missing, from another context, or profiling");
    CK(cudaSetDevice(ctx->device), ctx);
    std::lock_guard<std::mutex> lk(ctx->group_mu);
    // the batches' uploads (on their own streams) must be complete before the
    // streams join a capture or the graph reads their buffers
    for (int i = 0; i < nb; i++) CK(cudaStreamSynchronize(batches[i]->s), ctx);
    for (int i = 0; i < nb; i++) spec_scratch(batches[i]);
    cuspx_ctx::GroupGraph *hit = nullptr;
    for (auto &g : ctx->groups) {
        if ((int)g.batches.size() != nb) continue;
        bool same = true;
        for (int i = 0; i < nb && same; i++) {
            cuspx_batch *b = batches[i];
            same = g.batches[i] == b && g.counts[i] == b->count && g.long_msgs[i] == b->long_msgs &&
                   memcmp(&g.tunes[i], &effective_tuning(ctx, b->set, b->op, b->count), sizeof(Tuning)) == 0;
        }
        if (same) hit = &g;
    }
    if (!hit) {
        cuspx_ctx::GroupGraph gg;
        gg.batches.assign(batches, batches + nb);
        for (int i = 0; i < nb; i++) {
            gg.counts.push_back(batches[i]->count);
            gg.long_msgs.push_back(batches[i]->long_msgs);
            gg.tunes.push_back(effective_tuning(ctx, batches[i]->set, batches[i]->op, batches[i]->count));
        }
        CK(cudaStreamCreateWithFlags(&gg.origin, cudaStreamNonBlocking), ctx);
        cudaEventCreate(&gg.e0);
        cudaEventCreate(&gg.e1);
        std::vector<cudaEvent_t> fork(nb + 1), join(nb);
        for (auto &e : fork) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        for (auto &e : join) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(gg.origin, cudaStreamCaptureModeThreadLocal), ctx);
        cudaEventRecord(fork[0], gg.origin);
        for (int i = 0; i < nb; i++) {
            cudaStreamWaitEvent(batches[i]->s, fork[0], 0);
            launch_seq(batches[i], nullptr);
            cudaEventRecord(join[i], batches[i]->s);
            cudaStreamWaitEvent(gg.origin, join[i], 0);
        }
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(gg.origin, &graph);
        for (auto &e : fork) cudaEventDestroy(e);
        for (auto &e : join) cudaEventDestroy(e);
        if (le != cudaSuccess) return cuda_fail(ctx, le, "group launch during capture");
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "group cudaStreamEndCapture");
        cudaError_t ie = cudaGraphInstantiate(&gg.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_fail(ctx, ie, "group cudaGraphInstantiate");
        if (ctx->groups.size() >= 16) {
            auto &old = ctx->groups.front();
            cudaStreamSynchronize(old.origin);
            cudaGraphExecDestroy(old.exec);
            cudaEventDestroy(old.e0);
            cudaEventDestroy(old.e1);
            cudaStreamDestroy(old.origin);
            ctx->groups.erase(ctx->groups.begin());
        }
        ctx->groups.push_back(gg);
        hit = &ctx->groups.back();
    }
    CK(cudaEventRecord(hit->e0, hit->origin), ctx);
    CK(cudaGraphLaunch(hit->exec, hit->origin), ctx);
    CK(cudaEventRecord(hit->e1, hit->origin), ctx);
    CK(cudaStreamSynchronize(hit->origin), ctx);
    if (ms) CK(cudaEventElapsedTime(ms, hit->e0, hit->e1), ctx);
    for (int i = 0; i < nb; i++) batches[i]->ran = false;
    return CUSPX_OK;
}

}  // extern "C"
