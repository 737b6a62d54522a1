// serve.cu -- the serving face (include/cuspx_serve.h): resident keys,
// continuous batching over several in-flight launches per (operation, set),
// memory-budgeted admission, per-request latency, and an open-loop Poisson
// load generator.
//
// Threads: callers submit and wait under one mutex; three scheduler threads,
// one per message-length class, own every CUDA call on the serving batches
// of their groups (pack into pinned staging, upload, launch, asynchronous
// download, completion by event query), so a batch object is only ever
// touched by one thread.  Packing a long-message launch copies up to 64 MiB
// into pinned staging; with one scheduler, short launches and completions
// waited behind that host work.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cuspx.h"
#include "../../include/cuspx_serve.h"
#include "spx_kernels.cuh"
#include "spx_sets.h"

namespace cuspx {
SetParams make_params(const SetDesc &s);
int batch_share_stream(cuspx_batch *b, cudaStream_t s);
void batch_use_stream(cuspx_batch *b, cudaStream_t s);
void batch_direct_launch(cuspx_batch *b, bool on);
}
using namespace cuspx;
using Clock = std::chrono::steady_clock;

namespace {

struct Req {
    uint64_t ticket = 0;
    int op = 0, set = 0;
    uint32_t key = 0;
    const uint8_t *msg = nullptr;
    size_t mlen = 0;
    std::vector<uint8_t> msg_own;
    const uint8_t *sig = nullptr;
    size_t siglen = 0;
    std::vector<uint8_t> sig_own;
    std::vector<uint8_t> out;
    int32_t status = 0;
    int32_t expect = 1;     // load generator: expected verdict (1 = none)
    bool done = false;
    bool waiting = false;   // a thread is in cuspx_serve_wait on this request
    unsigned flags = 0;
    size_t admit_bytes = 0; // device bytes counted against the budget at submit
    double work_ops = 0;    // estimated integer ops of its hashing
    Clock::time_point t0, t1;
};

struct KeyTable {
    size_t cap = 0, n = 0;
    uint8_t *d_sk = nullptr, *d_pk = nullptr;
    std::vector<uint8_t> has_sk;
};

struct Slot {
    cuspx_batch *b = nullptr;
    size_t cap = 0, msg_cap = 0;
    double work = 0;   // estimated ops of the launch in flight
    uint8_t *h_msg = nullptr;
    uint64_t *h_off = nullptr, *h_len = nullptr, *h_siglen = nullptr;
    uint32_t *h_kidx = nullptr;
    uint8_t *h_aux = nullptr, *h_out = nullptr;
    int32_t *h_status = nullptr;
    cudaEvent_t ev = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;   // device time of the launch
    int stream = -1;   // index in the class's pool of the current launch's stream
    bool busy = false;
    size_t bytes = 0;
    std::vector<Req *> reqs;
};

// Requests are grouped per (operation, set, length class).  Message hashing
// is serial over the message on one thread (or one two-warp pair), and a
// launch ends with its longest message, so requests are launched with others
// of similar length: up to 16 KiB (<= 0.3 ms of hashing), up to 128 KiB
// (<= 4 ms) and longer (up to ~33 ms per 1 MiB sign).  A 64 KiB request thus
// never waits for a 1 MiB one in its own launch.
constexpr int kClasses = 3;
constexpr size_t kShortMsg = 16384;
constexpr size_t kMidMsg = 131072;
// Message area of one launch: a full batch of short messages, 32 MiB of
// middle-class or 64 MiB of long messages.  Slots are created once at this
// size and never re-created (freeing device or pinned memory waits for the
// whole device).
constexpr size_t kMidLaunchBytes = (size_t)32 << 20;
constexpr size_t kLongLaunchBytes = (size_t)64 << 20;
// a long-class launch holds at most 64 MiB / 128 KiB messages
constexpr size_t kLongItems = kLongLaunchBytes / kMidMsg;
// Streams per length class.  Each launch runs on the stream of its class's
// pool with the fewest launches in flight.  The device has a fixed number of
// hardware work queues (32 requested, see cuspx_create); with one stream per
// slot -- 2 operations x sets x classes x slots of them -- streams outnumber
// the queues and a short launch could wait in a queue behind a 1 MiB
// message-hashing kernel of another class (measured: <= 1 KiB sign p99 of
// 95 ms at 20k req/s of the mixed 16 B..1 MiB stream, 8.8 ms with pools).
// The long class gets the most streams: its launches last ~33-46 ms (serial
// hashing of a 1 MiB message) while using few SMs, so many must overlap.
constexpr int kClassStreams[kClasses] = {8, 8, 16};
// launch slots per group: max_inflight, and at least kLongSlots for long
// messages (whose launches are long but light)
constexpr int kLongSlots = 6;

int class_of(size_t mlen) { return mlen <= kShortMsg ? 0 : (mlen <= kMidMsg ? 1 : 2); }

struct Group {
    int op = 0, set = 0, cls = 0;
    std::deque<Req *> pending;
    std::vector<Slot *> slots;
    size_t per_item = 0;
    double item_ops = 0;   // estimated integer ops of one request, message hashing excluded
    SetParams P{};
};

// Expected hash units of one operation of a set, message hashing excluded,
// counted the way the reference runs it (crypto_sign_signature,
// crypto_sign_verify): the model the benchmark's roofline fractions use.
// The WOTS+ digit sum is its expectation over random messages: 7.5 per
// message digit, about 7.5 for the two low checksum digits and 15n / 256
// for the top one.
void op_units(const SetDesc &sd, double &sign, double &verify, double &ops_per_unit) {
    const int n = sd.n, hp = sd.h / sd.d, a = sd.a, k = sd.k, d = sd.d, ln = 2 * n + 3;
    const bool shake = sd.hash == 1, robust = sd.robust != 0;
    auto th = [&](int m) -> double {
        if (shake) return (n + 32 + m * n) / 136 + 1 + (robust ? (m * n + 135) / 136 : 0);
        return (22 + m * n + 9 + 63) / 64 + (robust ? ((m * n + 31) / 32) * ((n + 26 + 9 + 63) / 64) : 0);
    };
    const double F = th(1), H = th(2), prf = 1, seed = shake ? 0 : 1;
    const double leaf = ln * (prf + 15 * F) + th(ln);
    const double xmss = (double)(1 << hp) * leaf + ((1 << hp) - 1) * H;
    const double e = 2 * n * 7.5 + 7.5 + 7.5 + 15.0 * n / 256.0;
    sign = seed + k * (prf + (double)(1 << a) * (prf + F) + ((1 << a) - 1) * H) + th(k) + d * xmss +
           d * (ln * prf + e * F);
    verify = seed + k * (F + a * H) + th(k) + d * (th(ln) + hp * H) + d * (ln * 15 - e) * F;
    ops_per_unit = shake ? 4560.0 : 1384.0;
}

// Latency histogram: bin i holds [2^(i/64), 2^((i+1)/64)) microseconds
// (1.1% wide), from 1 us to 2^31 us; a percentile is read as the
// geometric middle of its bin.  Fixed memory, O(bins) per read.
struct LatHist {
    static constexpr int kPerOctave = 64, kBins = 64 * 31;
    std::vector<uint64_t> bins = std::vector<uint64_t>(kBins, 0);
    uint64_t n = 0;
    void add(double us) {
        int i = us <= 1.0 ? 0 : (int)std::floor(std::log2(us) * kPerOctave);
        bins[std::min(std::max(i, 0), kBins - 1)]++;
        n++;
    }
    // value of the sample of rank round(q (n - 1)) in sorted order
    double pct(double q) const {
        if (!n) return 0.0;
        const uint64_t k = (uint64_t)std::min<double>((double)(n - 1), std::floor(q * (double)(n - 1) + 0.5));
        uint64_t cum = 0;
        for (int i = 0; i < kBins; i++) {
            cum += bins[i];
            if (cum > k) return std::exp2((i + 0.5) / kPerOctave);
        }
        return std::exp2((double)kBins / kPerOctave);
    }
    void clear() {
        std::fill(bins.begin(), bins.end(), 0);
        n = 0;
    }
};

// Hash units of a request's message hashing (SHA-256 compressions or
// Keccak-f[1600] permutations): H_msg for verify, PRF_msg and H_msg for
// sign (hash_sha256.cu:99-145, :200-262; hash_shake256.cu:64-77, :96-130).
double msg_units(int op, const SetDesc &sd, const SetParams &P, uint64_t mlen) {
    const uint64_t n = sd.n;
    if (sd.hash == 0) {
        // SHA256(R || PK || m), then MGF1 blocks of 32 digest bytes
        const uint64_t h = (3 * n + mlen + 9 + 63) / 64 + (P.dgst_bytes + 31) / 32;
        // HMAC: ipad block, optrand || m, then opad block and the inner digest
        return (double)(op == CUSPX_OP_VERIFY ? h : h + 3 + (n + mlen + 9 + 63) / 64);
    }
    const uint64_t h = (3 * n + mlen) / 136 + 1;
    return (double)(op == CUSPX_OP_VERIFY ? h : h + (2 * n + mlen) / 136 + 1);
}

}  // namespace

struct cuspx_server {
    cuspx_ctx *ctx = nullptr;
    cuspx_serve_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_sched[kClasses], cv_done;   // cv_sched[length class]
    std::thread th[kClasses];
    bool stop = false;
    std::vector<KeyTable> keys;
    std::vector<Group> groups;   // index ((op - 1) * kNumSets + set) * kClasses + class
    std::unordered_map<uint64_t, Req *> live;
    uint64_t next_ticket = 1;
    size_t pending_total = 0, pending_bytes = 0, bytes_inflight = 0, bytes_peak = 0;
    double work_queued = 0;   // estimated ops of the requests pending or in flight
    uint64_t submitted = 0, completed = 0, refused = 0, failed = 0, launches = 0, batched = 0;
    uint64_t sign_done = 0, verify_done = 0, wrong = 0;
    double launch_ms_sum = 0, launch_ms_max = 0;
    LatHist lat_sign, lat_verify;
    LatHist lat_bucket[2][3];   // [sign, verify][<= 1 KiB, <= 64 KiB, > 64 KiB]
    std::vector<cudaStream_t> streams[kClasses];   // per-class stream pools
    std::vector<int> stream_load[kClasses];         // launches in flight per pooled stream (under mu)
    uint64_t done_by_set[2][kNumSets] = {};   // [sign, verify][set]
    double msg_units_by_set[kNumSets] = {};
    Clock::time_point last_done;
    Group &group(int op, int set, int cls) { return groups[((op - 1) * kNumSets + set) * kClasses + cls]; }
};

static int len_bucket(size_t mlen) { return mlen <= 1024 ? 0 : (mlen <= 65536 ? 1 : 2); }

static size_t item_bytes(int op, const SetParams &P) {
    const size_t n = P.n;
    size_t b = sizeof(SignWork) + P.k * n + 64;
    if (op == CUSPX_OP_SIGN)
        b += P.sig_bytes + n + (size_t)P.d * ((size_t)1 << P.hp) * n + P.d * n + (size_t)P.d * P.len * 16 * n;
    else   // signature, its length, WOTS+ public key, root, sorted-verify bucket entries
        b += P.sig_bytes + 8 + (size_t)P.len * n + n + 16 * (size_t)P.len * sizeof(uint32_t);
    return b;
}

static void free_slot(Slot *sl) {
    if (sl->b) cuspx_batch_destroy(sl->b);
    cudaFreeHost(sl->h_msg);
    cudaFreeHost(sl->h_off);
    cudaFreeHost(sl->h_len);
    cudaFreeHost(sl->h_siglen);
    cudaFreeHost(sl->h_kidx);
    cudaFreeHost(sl->h_aux);
    cudaFreeHost(sl->h_out);
    cudaFreeHost(sl->h_status);
    if (sl->ev) cudaEventDestroy(sl->ev);
    if (sl->ev_start) cudaEventDestroy(sl->ev_start);
    if (sl->ev_end) cudaEventDestroy(sl->ev_end);
    delete sl;
}

static size_t class_msg_bytes(const cuspx_server *s, const Group &g) {
    return g.cls == 2 ? kLongLaunchBytes
                      : (g.cls == 1 ? kMidLaunchBytes : (size_t)s->cfg.max_batch * (kShortMsg + 16));
}
static size_t class_items(const cuspx_server *s, const Group &g) {
    return g.cls == 2 ? std::min<size_t>(s->cfg.max_batch, kLongItems) : (size_t)s->cfg.max_batch;
}
static int class_slots(const cuspx_server *s, const Group &g) {
    return g.cls == 2 ? std::max(s->cfg.max_inflight, kLongSlots) : s->cfg.max_inflight;
}

// Create a slot's batch and pinned staging once, at the full size of its
// group (the class's items and message area).
static bool size_slot(cuspx_server *s, Group &g, Slot *sl) {
    const SetParams &P = g.P;
    if (sl->b) return true;
    const size_t cap = class_items(s, g);
    const size_t msg_cap = class_msg_bytes(s, g);
    if (cuspx_batch_create(s->ctx, g.op, g.set, cap, msg_cap, 1, &sl->b) != CUSPX_OK) return false;
    batch_direct_launch(sl->b, true);   // no graph instantiation while serving
    batch_share_stream(sl->b, s->streams[g.cls][0]);   // the launch picks its stream
    const KeyTable &kt = s->keys[g.set];
    cuspx_batch_bind_keys(sl->b, g.op == CUSPX_OP_SIGN ? kt.d_sk : kt.d_pk, kt.cap);
    auto host = [](void **p, size_t bytes) { return cudaMallocHost(p, std::max<size_t>(bytes, 16)) == cudaSuccess; };
    bool ok = host((void **)&sl->h_msg, msg_cap + 64) && host((void **)&sl->h_off, cap * 8) &&
              host((void **)&sl->h_len, cap * 8) && host((void **)&sl->h_siglen, cap * 8) &&
              host((void **)&sl->h_kidx, cap * 4) &&
              host((void **)&sl->h_aux, g.op == CUSPX_OP_VERIFY ? cap * P.sig_bytes : 16) &&
              host((void **)&sl->h_out, g.op == CUSPX_OP_SIGN ? cap * P.sig_bytes : 16) &&
              host((void **)&sl->h_status, cap * 4);
    cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming);
    cudaEventCreate(&sl->ev_start);
    cudaEventCreate(&sl->ev_end);
    sl->cap = cap;
    sl->msg_cap = msg_cap;
    return ok;
}

// pack requests into the slot's pinned staging and launch asynchronously
static bool launch_slot(cuspx_server *s, Group &g, Slot *sl) {
    const SetParams &P = g.P;
    if (!size_slot(s, g, sl)) return false;
    // the slot is idle (its last launch completed): move it to the stream
    // chosen for this launch without waiting for anything
    cudaStream_t st = s->streams[g.cls][sl->stream];
    batch_use_stream(sl->b, st);
    cudaEventRecord(sl->ev_start, st);
    size_t off = 0;
    for (size_t i = 0; i < sl->reqs.size(); i++) {
        Req *r = sl->reqs[i];
        sl->h_off[i] = off;
        sl->h_len[i] = r->mlen;
        sl->h_kidx[i] = r->key;
        if (r->mlen) memcpy(sl->h_msg + off, r->msg, r->mlen);
        off += (r->mlen + 15) & ~(size_t)15;
        if (g.op == CUSPX_OP_VERIFY) {
            uint8_t *row = sl->h_aux + i * P.sig_bytes;
            const size_t take = std::min<size_t>(r->siglen, P.sig_bytes);
            memcpy(row, r->sig, take);
            if (take < (size_t)P.sig_bytes) memset(row + take, 0, P.sig_bytes - take);
            sl->h_siglen[i] = r->siglen;
        }
    }
    const size_t cnt = sl->reqs.size();
    if (cuspx_batch_upload(sl->b, cnt, nullptr, 0, sl->h_kidx, sl->h_msg, off, sl->h_off, sl->h_len,
                           g.op == CUSPX_OP_VERIFY ? sl->h_aux : nullptr,
                           g.op == CUSPX_OP_VERIFY ? sl->h_siglen : nullptr) != CUSPX_OK)
        return false;
    if (cuspx_batch_run(sl->b) != CUSPX_OK) return false;
    if (cuspx_batch_download_async(sl->b, g.op == CUSPX_OP_SIGN ? sl->h_out : nullptr, nullptr, sl->h_status) !=
        CUSPX_OK)
        return false;
    cudaEventRecord(sl->ev_end, st);
    return cudaEventRecord(sl->ev, st) == cudaSuccess;
}

// mark a slot's requests done (called with the lock held)
static void finish_slot(cuspx_server *s, Group &g, Slot *sl, bool ok) {
    const SetParams &P = g.P;
    const auto now = Clock::now();
    float lms = 0;
    if (ok && sl->ev_start && cudaEventElapsedTime(&lms, sl->ev_start, sl->ev_end) == cudaSuccess) {
        s->launch_ms_sum += lms;
        s->launch_ms_max = std::max<double>(s->launch_ms_max, lms);
    }
    for (size_t i = 0; i < sl->reqs.size(); i++) {
        Req *r = sl->reqs[i];
        r->status = ok ? sl->h_status[i] : -3;
        if (!ok) s->failed++;
        if (g.op == CUSPX_OP_SIGN && ok && !(r->flags & CUSPX_SUBMIT_DETACH))
            r->out.assign(sl->h_out + i * P.sig_bytes, sl->h_out + (i + 1) * P.sig_bytes);
        r->t1 = now;
        r->done = true;
        const double us = std::chrono::duration<double, std::micro>(now - r->t0).count();
        const int o = g.op == CUSPX_OP_SIGN ? 0 : 1;
        if (o == 0) {
            s->lat_sign.add(us);
            s->sign_done++;
        } else {
            s->lat_verify.add(us);
            s->verify_done++;
        }
        s->lat_bucket[o][len_bucket(r->mlen)].add(us);
        if (ok) {
            s->done_by_set[o][g.set]++;
            s->msg_units_by_set[g.set] += msg_units(g.op, kSets[g.set], P, r->mlen);
        }
        if (r->expect != 1 && r->status != r->expect) s->wrong++;
        s->completed++;
        if (r->flags & CUSPX_SUBMIT_DETACH) {
            s->live.erase(r->ticket);
            delete r;
        }
    }
    s->last_done = now;
    sl->reqs.clear();
    if (sl->stream >= 0) s->stream_load[g.cls][sl->stream]--;
    sl->stream = -1;
    s->work_queued -= sl->work;
    if (s->work_queued < 0) s->work_queued = 0;
    sl->work = 0;
    s->bytes_inflight -= sl->bytes;
    sl->bytes = 0;
    sl->busy = false;
}

// Scheduler of the groups of one length class (lc).
static void scheduler(cuspx_server *s, int lc) {
    cudaSetDevice(s->device);
    const auto window = std::chrono::microseconds(s->cfg.window_us);
    const auto drain_deadline_len = std::chrono::seconds(60);
    Clock::time_point drain_deadline{};
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        // ---- retire finished launches ----
        bool any_busy = false;
        size_t class_pending = 0;
        for (Group &g : s->groups) {
            if (g.cls != lc) continue;
            class_pending += g.pending.size();
            for (Slot *sl : g.slots) {
                if (!sl->busy) continue;
                cudaError_t e = cudaEventQuery(sl->ev);
                if (e == cudaErrorNotReady) {
                    any_busy = true;
                    continue;
                }
                finish_slot(s, g, sl, e == cudaSuccess);
                s->cv_done.notify_all();
            }
        }
        if (s->stop) {
            if (drain_deadline == Clock::time_point{}) drain_deadline = Clock::now() + drain_deadline_len;
            if ((!any_busy && class_pending == 0) || Clock::now() > drain_deadline) break;
        }
        // ---- admit new launches ----
        const auto now = Clock::now();
        Clock::time_point next_wake = now + std::chrono::microseconds(50);
        for (Group &g : s->groups) {
            if (g.cls != lc) continue;
            while (!g.pending.empty()) {
                int inflight = 0;
                Slot *free_sl = nullptr;
                for (Slot *sl : g.slots) {
                    if (sl->busy) inflight++;
                    else if (!free_sl) free_sl = sl;
                }
                const size_t items = class_items(s, g);
                const bool full = g.pending.size() >= items;
                const bool waited = now - g.pending.front()->t0 >= window;
                if (!(full || waited || inflight == 0)) {
                    next_wake = std::min(next_wake, g.pending.front()->t0 + window);
                    break;
                }
                if (!free_sl) {
                    if ((int)g.slots.size() >= class_slots(s, g)) break;
                    free_sl = new Slot();
                    g.slots.push_back(free_sl);
                }
                // take as many as fit the launch's items and message area
                // (their device bytes were admitted against the budget when
                // they were submitted, so pending + in-flight stays within it)
                size_t n = 0, bytes = 0, mbytes = 0;
                double work = 0;
                const size_t mcap = class_msg_bytes(s, g);
                const double wcap = s->cfg.max_launch_ms > 0 ? s->cfg.max_launch_ms * 1e-3 * s->cfg.gpu_ops_per_s : 0;
                for (Req *r : g.pending) {
                    if (n == items) break;
                    const size_t m16 = (r->mlen + 15) & ~(size_t)15;
                    if (mbytes + m16 > mcap) break;
                    if (wcap > 0 && n > 0 && work + r->work_ops > wcap) break;
                    mbytes += m16;
                    bytes += r->admit_bytes;
                    work += r->work_ops;
                    n++;
                }
                if (n == 0) break;
                for (size_t i = 0; i < n; i++) {
                    free_sl->reqs.push_back(g.pending.front());
                    g.pending.pop_front();
                }
                s->pending_total -= n;
                s->pending_bytes -= bytes;
                free_sl->busy = true;
                free_sl->bytes = bytes;
                free_sl->work = work;
                {
                    // the class's least loaded stream
                    std::vector<int> &load = s->stream_load[g.cls];
                    int best = 0;
                    for (int i = 1; i < (int)load.size(); i++)
                        if (load[i] < load[best]) best = i;
                    load[best]++;
                    free_sl->stream = best;
                }
                s->bytes_inflight += bytes;
                s->bytes_peak = std::max(s->bytes_peak, s->bytes_inflight);
                s->launches++;
                s->batched += n;
                lk.unlock();
                const bool ok = launch_slot(s, g, free_sl);
                lk.lock();
                if (!ok) {
                    finish_slot(s, g, free_sl, false);
                    s->cv_done.notify_all();
                }
            }
        }
        s->cv_sched[lc].wait_until(lk, next_wake);
    }
}

extern "C" {

int cuspx_serve_create(cuspx_ctx *ctx, const cuspx_serve_config *cfg, cuspx_server **out) {
    if (!ctx || !out) return CUSPX_EINVAL;
    cuspx_server *s = new cuspx_server();
    s->ctx = ctx;
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.mem_budget) s->cfg.mem_budget = (size_t)8 << 30;
    if (s->cfg.max_batch <= 0) s->cfg.max_batch = 1024;
    if (s->cfg.max_inflight <= 0) s->cfg.max_inflight = 3;
    if (s->cfg.window_us <= 0) s->cfg.window_us = 500;
    if (s->cfg.max_keys <= 0) s->cfg.max_keys = 4096;
    if (!s->cfg.max_queue) s->cfg.max_queue = 1u << 20;
    cudaGetDevice(&s->device);
    if (s->cfg.gpu_ops_per_s <= 0 && (s->cfg.max_queue_ms > 0 || s->cfg.max_launch_ms > 0)) {
        // 60% of the SHA-256-round peak: about what the served three-set
        // stream reaches at saturation
        double peak = 0;
        float ms = 0;
        if (cuspx_int_peak_mix(s->device, 1024, 1, &peak, &ms) != CUSPX_OK || peak <= 0) peak = 2e13;
        s->cfg.gpu_ops_per_s = 0.6 * peak;
    }
    s->keys.resize(kNumSets);
    s->groups.resize(2 * kNumSets * kClasses);
    for (int op = 1; op <= 2; op++)
        for (int set = 0; set < kNumSets; set++)
            for (int lc = 0; lc < kClasses; lc++) {
                Group &g = s->group(op, set, lc);
                g.op = op;
                g.set = set;
                g.cls = lc;
                g.P = make_params(kSets[set]);
                g.per_item = item_bytes(op, g.P);
                double su, vu, opu;
                op_units(kSets[set], su, vu, opu);
                g.item_ops = (op == CUSPX_OP_SIGN ? su : vu) * opu;
            }
    // short-message launches run ahead of middle ones, those ahead of long
    // ones on the GPU (lo is the least urgent priority, hi the most)
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    for (int lc = 0; lc < kClasses; lc++) {
        const int prio = lc == 0 ? hi : (lc == 1 ? (lo + hi) / 2 : lo);
        for (int i = 0; i < kClassStreams[lc]; i++) {
            cudaStream_t st = nullptr;
            if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio) != cudaSuccess) {
                for (auto &p : s->streams)
                    for (cudaStream_t x : p) cudaStreamDestroy(x);
                delete s;
                return CUSPX_ECUDA;
            }
            s->streams[lc].push_back(st);
        }
        s->stream_load[lc].assign(s->streams[lc].size(), 0);
    }
    for (int lc = 0; lc < kClasses; lc++) s->th[lc] = std::thread(scheduler, s, lc);
    *out = s;
    return CUSPX_OK;
}

void cuspx_serve_destroy(cuspx_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    for (int lc = 0; lc < kClasses; lc++) s->cv_sched[lc].notify_all();
    for (int lc = 0; lc < kClasses; lc++)
        if (s->th[lc].joinable()) s->th[lc].join();
    for (Group &g : s->groups) {
        for (Slot *sl : g.slots) {
            if (sl->busy && sl->b) cuspx_batch_sync(sl->b);
            free_slot(sl);
        }
        for (Req *r : g.pending) delete r;
    }
    for (auto &kv : s->live)
        if (kv.second->done) delete kv.second;   // completed but never waited for
    for (KeyTable &kt : s->keys) {
        cudaFree(kt.d_sk);
        cudaFree(kt.d_pk);
    }
    for (auto &p : s->streams)
        for (cudaStream_t x : p) cudaStreamDestroy(x);
    delete s;
}

// The set's resident key table, allocated once at max_keys rows (so the
// device address the slots are bound to never changes); lock held.
static int ensure_table(cuspx_server *s, int set) {
    KeyTable &kt = s->keys[set];
    if (kt.d_sk) return CUSPX_OK;
    const size_t n = kSets[set].n;
    kt.cap = s->cfg.max_keys;
    if (cudaMalloc(&kt.d_sk, kt.cap * 4 * n) != cudaSuccess || cudaMalloc(&kt.d_pk, kt.cap * 2 * n) != cudaSuccess)
        return CUSPX_ENOMEM;
    cudaMemset(kt.d_sk, 0, kt.cap * 4 * n);
    cudaMemset(kt.d_pk, 0, kt.cap * 2 * n);
    return CUSPX_OK;
}

static int add_rows(cuspx_server *s, int set, size_t count, const uint8_t *rows, bool secret, uint32_t *first) {
    if (!s || set < 0 || set >= kNumSets || (count && !rows)) return CUSPX_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    KeyTable &kt = s->keys[set];
    const size_t n = kSets[set].n;
    if (int rc = ensure_table(s, set)) return rc;
    if (kt.n + count > kt.cap) return CUSPX_ENOMEM;
    for (size_t i = 0; i < count; i++) {
        const uint8_t *r = rows + i * (secret ? 4 * n : 2 * n);
        if (secret) {
            if (cudaMemcpy(kt.d_sk + (kt.n + i) * 4 * n, r, 4 * n, cudaMemcpyHostToDevice)) return CUSPX_ECUDA;
            if (cudaMemcpy(kt.d_pk + (kt.n + i) * 2 * n, r + 2 * n, 2 * n, cudaMemcpyHostToDevice)) return CUSPX_ECUDA;
        } else {
            if (cudaMemcpy(kt.d_pk + (kt.n + i) * 2 * n, r, 2 * n, cudaMemcpyHostToDevice)) return CUSPX_ECUDA;
        }
        kt.has_sk.push_back(secret ? 1 : 0);
    }
    if (first) *first = (uint32_t)kt.n;
    kt.n += count;
    return CUSPX_OK;
}

// Create every launch slot of (op, set) -- all length classes, max_inflight
// each -- now instead of on first use: a slot's device batch and pinned
// staging (64 MiB for long messages) take milliseconds to allocate, and
// device allocation can wait for work already on the GPU, so creating them
// while requests flow puts that time on the requests' latency.
int cuspx_serve_prepare(cuspx_server *s, int op, int set) {
    if (!s || (op != CUSPX_OP_SIGN && op != CUSPX_OP_VERIFY) || set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    if (cudaSetDevice(s->device) != cudaSuccess) return CUSPX_ECUDA;
    std::lock_guard<std::mutex> lk(s->mu);
    if (int rc = ensure_table(s, set)) return rc;
    for (int lc = 0; lc < kClasses; lc++) {
        Group &g = s->group(op, set, lc);
        while ((int)g.slots.size() < class_slots(s, g)) {
            Slot *sl = new Slot();
            if (!size_slot(s, g, sl)) {
                free_slot(sl);
                return CUSPX_ENOMEM;
            }
            g.slots.push_back(sl);
        }
    }
    return CUSPX_OK;
}

int cuspx_serve_add_keys(cuspx_server *s, int set, size_t count, const uint8_t *sks, uint32_t *first_id) {
    return add_rows(s, set, count, sks, true, first_id);
}

int cuspx_serve_add_pubkeys(cuspx_server *s, int set, size_t count, const uint8_t *pks, uint32_t *first_id) {
    return add_rows(s, set, count, pks, false, first_id);
}

static int submit(cuspx_server *s, int op, int set, uint32_t key_id, const uint8_t *msg, size_t mlen,
                  const uint8_t *sig, size_t siglen, unsigned flags, int32_t expect, uint64_t *ticket) {
    if (!s || (op != CUSPX_OP_SIGN && op != CUSPX_OP_VERIFY) || set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    if (mlen && !msg) return CUSPX_EINVAL;
    if (op == CUSPX_OP_VERIFY && siglen && !sig) return CUSPX_EINVAL;
    Req *r = new Req();
    r->op = op;
    r->set = set;
    r->key = key_id;
    r->flags = flags;
    r->expect = expect;
    if (flags & CUSPX_SUBMIT_BORROW) {
        r->msg = msg;
        r->sig = sig;
    } else {
        r->msg_own.assign(msg, msg + mlen);
        r->msg = r->msg_own.data();
        if (op == CUSPX_OP_VERIFY) {
            r->sig_own.assign(sig, sig + siglen);
            r->sig = r->sig_own.data();
        }
    }
    r->mlen = mlen;
    r->siglen = op == CUSPX_OP_VERIFY ? siglen : 0;
    std::unique_lock<std::mutex> lk(s->mu);
    const KeyTable &kt = s->keys[set];
    Group &g = s->group(op, set, class_of(mlen));
    r->admit_bytes = g.per_item + ((mlen + 15) & ~(size_t)15);
    {
        double su, vu, opu;
        op_units(kSets[set], su, vu, opu);
        r->work_ops = g.item_ops + msg_units(op, kSets[set], g.P, mlen) * opu;
    }
    int rc = CUSPX_OK;
    if (s->stop) rc = CUSPX_EBUSY;
    else if (key_id >= kt.n || (op == CUSPX_OP_SIGN && !kt.has_sk[key_id])) rc = CUSPX_EINVAL;
    else if (r->admit_bytes > s->cfg.mem_budget) rc = CUSPX_ENOMEM;   // could never be admitted
    else if (mlen + 16 > kLongLaunchBytes) rc = CUSPX_ETOOBIG;
    else if (s->pending_total >= s->cfg.max_queue) rc = CUSPX_EBUSY;
    // admission by device-memory budget: the bytes of everything pending or
    // in flight, this request included
    else if (s->pending_bytes + s->bytes_inflight + r->admit_bytes > s->cfg.mem_budget) rc = CUSPX_EBUSY;
    // admission by queued work: what is pending or in flight, in ms of the
    // device's capacity (a request is admitted into an empty queue whatever
    // its size)
    else if (s->cfg.max_queue_ms > 0 && s->work_queued > 0 &&
             (s->work_queued + r->work_ops) / s->cfg.gpu_ops_per_s * 1e3 > s->cfg.max_queue_ms)
        rc = CUSPX_EBUSY;
    if (rc != CUSPX_OK) {
        s->refused++;
        lk.unlock();
        delete r;
        return rc;
    }
    r->ticket = s->next_ticket++;
    r->t0 = Clock::now();
    s->live[r->ticket] = r;
    g.pending.push_back(r);
    s->pending_total++;
    s->pending_bytes += r->admit_bytes;
    s->work_queued += r->work_ops;
    s->submitted++;
    if (ticket) *ticket = r->ticket;
    const bool kick = g.pending.size() == 1 || g.pending.size() >= class_items(s, g);
    lk.unlock();
    if (kick) s->cv_sched[g.cls].notify_one();
    return CUSPX_OK;
}

int cuspx_serve_submit(cuspx_server *s, int op, int set, uint32_t key_id, const uint8_t *msg, size_t mlen,
                       const uint8_t *sig, size_t siglen, unsigned flags, uint64_t *ticket) {
    return submit(s, op, set, key_id, msg, mlen, sig, siglen, flags, 1, ticket);
}

int cuspx_serve_wait(cuspx_server *s, uint64_t ticket, long timeout_us, uint8_t *sig_out, int32_t *status,
                     double *latency_us) {
    if (!s) return CUSPX_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return CUSPX_EINVAL;
    Req *r = it->second;
    // a detached request is freed by its completion, and a request has one
    // waiter: a second one would wake to a freed request
    if ((r->flags & CUSPX_SUBMIT_DETACH) || r->waiting) return CUSPX_EINVAL;
    r->waiting = true;
    auto pred = [&] { return r->done; };
    if (timeout_us < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), pred)) {
        r->waiting = false;
        return CUSPX_ETIMEDOUT;
    }
    if (sig_out && !r->out.empty()) memcpy(sig_out, r->out.data(), r->out.size());
    if (status) *status = r->status;
    if (latency_us) *latency_us = std::chrono::duration<double, std::micro>(r->t1 - r->t0).count();
    s->live.erase(r->ticket);
    delete r;
    return CUSPX_OK;
}

int cuspx_serve_stats(cuspx_server *s, cuspx_serve_counters *st) {
    if (!s || !st) return CUSPX_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    {
        st->submitted = s->submitted;
        st->completed = s->completed;
        st->refused = s->refused;
        st->failed = s->failed;
        st->launches = s->launches;
        st->sign_done = s->sign_done;
        st->verify_done = s->verify_done;
        st->bytes_inflight = s->bytes_inflight;
        st->bytes_peak = s->bytes_peak;
        st->mean_batch = s->launches ? (double)s->batched / s->launches : 0.0;
        st->launch_ms_mean = s->launches ? s->launch_ms_sum / s->launches : 0.0;
        st->launch_ms_max = s->launch_ms_max;
    }
    st->sign_p50_us = s->lat_sign.pct(0.50);
    st->sign_p99_us = s->lat_sign.pct(0.99);
    st->verify_p50_us = s->lat_verify.pct(0.50);
    st->verify_p99_us = s->lat_verify.pct(0.99);
    for (int b = 0; b < 3; b++) {
        st->sign_p50_bucket_us[b] = s->lat_bucket[0][b].pct(0.50);
        st->sign_p99_bucket_us[b] = s->lat_bucket[0][b].pct(0.99);
        st->verify_p50_bucket_us[b] = s->lat_bucket[1][b].pct(0.50);
        st->verify_p99_bucket_us[b] = s->lat_bucket[1][b].pct(0.99);
        st->bucket_count[0][b] = s->lat_bucket[0][b].n;
        st->bucket_count[1][b] = s->lat_bucket[1][b].n;
    }
    return CUSPX_OK;
}

int cuspx_serve_reset_stats(cuspx_server *s) {
    if (!s) return CUSPX_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    s->submitted = s->completed = s->refused = s->failed = s->launches = s->batched = 0;
    s->sign_done = s->verify_done = s->wrong = 0;
    s->launch_ms_sum = s->launch_ms_max = 0;
    s->bytes_peak = s->bytes_inflight;
    s->lat_sign.clear();
    s->lat_verify.clear();
    for (auto &o : s->lat_bucket)
        for (auto &b : o) b.clear();
    memset(s->done_by_set, 0, sizeof(s->done_by_set));
    memset(s->msg_units_by_set, 0, sizeof(s->msg_units_by_set));
    return CUSPX_OK;
}

// ---------------------------------------------------------------------------
// open-loop Poisson load generator
// ---------------------------------------------------------------------------
int cuspx_serve_loadgen(cuspx_server *s, const cuspx_loadgen_config *c, cuspx_loadgen_result *out) {
    if (!s || !c || !out || c->nsets <= 0 || !c->sets || c->rate <= 0 || c->seconds <= 0 || c->keys_per_set == 0 ||
        c->min_len > c->max_len)
        return CUSPX_EINVAL;
    std::mt19937_64 rng(c->seed);
    const size_t buf_len = c->max_len + 4096;
    std::vector<uint8_t> buf(buf_len);
    for (auto &x : buf) x = (uint8_t)rng();
    const double lmin = std::log((double)std::max<uint64_t>(1, c->min_len));
    const double lmax = std::log((double)std::max<uint64_t>(1, c->max_len));
    auto draw_len = [&]() -> size_t {
        std::uniform_real_distribution<double> u(lmin, lmax);
        size_t L = (size_t)std::floor(std::exp(u(rng)));
        return std::min<size_t>(std::max<size_t>(L, c->min_len), c->max_len);
    };
    auto draw_off = [&](size_t L) -> size_t { return (size_t)(rng() % (buf_len - L + 1)); };

    // pre-signed pool per set for verify requests (and a corrupted twin of each)
    const int pool = std::max(1, c->pool);
    struct Entry {
        const uint8_t *m;
        size_t mlen;
        uint32_t key;
        std::vector<uint8_t> sig, bad;
    };
    std::vector<std::vector<Entry>> pools(c->nsets);
    for (int si = 0; si < c->nsets; si++) {
        const int set = c->sets[si];
        size_t sigb = 0;
        cuspx_set_sizes(set, nullptr, nullptr, &sigb, nullptr, nullptr);
        std::vector<uint64_t> tickets(pool);
        pools[si].resize(pool);
        int waited = 0;   // entries [0, waited) have their signatures
        auto wait_upto = [&](int upto) -> int {
            for (; waited < upto; waited++) {
                Entry &e = pools[si][waited];
                int32_t st = 0;
                int rc = cuspx_serve_wait(s, tickets[waited], 120000000L, e.sig.data(), &st, nullptr);
                if (rc || st) return rc ? rc : CUSPX_ECUDA;
            }
            return CUSPX_OK;
        };
        for (int i = 0; i < pool; i++) {
            Entry &e = pools[si][i];
            e.mlen = draw_len();
            e.m = buf.data() + draw_off(e.mlen);
            e.key = (uint32_t)(rng() % c->keys_per_set);
            e.sig.resize(sigb);
            int rc = submit(s, CUSPX_OP_SIGN, set, e.key, e.m, e.mlen, nullptr, 0, CUSPX_SUBMIT_BORROW, 1, &tickets[i]);
            if (rc == CUSPX_EBUSY) {   // over the admission budget: let the earlier ones finish
                if ((rc = wait_upto(i))) return rc;
                rc = submit(s, CUSPX_OP_SIGN, set, e.key, e.m, e.mlen, nullptr, 0, CUSPX_SUBMIT_BORROW, 1, &tickets[i]);
            }
            if (rc) return rc;
        }
        if (int rc = wait_upto(pool)) return rc;
        for (int i = 0; i < pool; i++) {
            Entry &e = pools[si][i];
            e.bad = e.sig;
            const size_t pos = (size_t)(rng() % sigb);
            e.bad[pos] ^= (uint8_t)(1u << (rng() % 8));
        }
    }
    cuspx_serve_reset_stats(s);

    std::exponential_distribution<double> gap(c->rate);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    uint64_t offered = 0, refused = 0;
    // sampled sign requests: kept (not detached) and copied out after the run
    struct Pick {
        uint64_t ticket;
        int set;
        uint32_t key;
        const uint8_t *m;
        size_t mlen, sigb;
    };
    std::vector<Pick> picks;
    uint64_t signs_offered = 0;
    size_t arena_used = 0;
    const auto t0 = Clock::now();
    double t_next = 0.0;
    while (true) {
        t_next += gap(rng);
        if (t_next >= c->seconds) break;
        const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(t_next));
        while (true) {
            auto now = Clock::now();
            if (now >= due) break;
            if (due - now > std::chrono::microseconds(200)) std::this_thread::sleep_for(due - now - std::chrono::microseconds(100));
            else std::this_thread::yield();
        }
        const int si = (int)(rng() % c->nsets);
        const int set = c->sets[si];
        int rc;
        offered++;
        if (U(rng) < c->verify_frac) {
            const Entry &e = pools[si][rng() % pool];
            const bool corrupt = U(rng) < c->corrupt_frac;
            const std::vector<uint8_t> &sg = corrupt ? e.bad : e.sig;
            rc = submit(s, CUSPX_OP_VERIFY, set, e.key, e.m, e.mlen, sg.data(), sg.size(),
                        CUSPX_SUBMIT_BORROW | CUSPX_SUBMIT_DETACH, corrupt ? -1 : 0, nullptr);
        } else {
            const size_t L = draw_len();
            const uint32_t key = (uint32_t)(rng() % c->keys_per_set);
            const uint8_t *m = buf.data() + draw_off(L);
            size_t sigb = 0;
            cuspx_set_sizes(set, nullptr, nullptr, &sigb, nullptr, nullptr);
            const bool pick = c->sample_every && c->samples && c->arena && signs_offered % c->sample_every == 0 &&
                              picks.size() < c->sample_max && arena_used + L + sigb <= c->arena_bytes;
            signs_offered++;
            uint64_t t = 0;
            rc = submit(s, CUSPX_OP_SIGN, set, key, m, L, nullptr, 0,
                        CUSPX_SUBMIT_BORROW | (pick ? 0u : CUSPX_SUBMIT_DETACH), 1, &t);
            if (pick && rc == CUSPX_OK) {
                picks.push_back(Pick{t, set, key, m, L, sigb});
                arena_used += L + sigb;
            }
        }
        if (rc) refused++;
    }
    // drain (bounded)
    const auto deadline = Clock::now() + std::chrono::seconds(120);
    {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_done.wait_until(lk, deadline, [&] { return s->completed >= offered - refused; });
    }
    cuspx_serve_counters st;
    cuspx_serve_stats(s, &st);
    double wall;
    uint64_t wrong;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        wall = std::chrono::duration<double>(s->last_done - t0).count();
        wrong = s->wrong;
        for (int si = 0; si < 8; si++) {
            const bool in = si < c->nsets;
            out->set_sign_done[si] = in ? s->done_by_set[0][c->sets[si]] : 0;
            out->set_verify_done[si] = in ? s->done_by_set[1][c->sets[si]] : 0;
            out->set_msg_units[si] = in ? s->msg_units_by_set[c->sets[si]] : 0.0;
        }
    }
    // the sampled signatures (every sampled request completed in the drain
    // above, or its wait runs out here)
    size_t at = 0;
    out->sampled = 0;
    for (const Pick &pk : picks) {
        cuspx_loadgen_sample &smp = c->samples[out->sampled];
        smp.set = pk.set;
        smp.key_id = pk.key;
        smp.mlen = pk.mlen;
        smp.msg_off = at;
        smp.sig_off = at + pk.mlen;
        smp.pad = 0;
        int32_t sst = -3;
        if (cuspx_serve_wait(s, pk.ticket, 10000000L, c->arena + smp.sig_off, &sst, nullptr) != CUSPX_OK) continue;
        if (pk.mlen) memcpy(c->arena + smp.msg_off, pk.m, pk.mlen);
        smp.status = sst;
        at += pk.mlen + pk.sigb;
        out->sampled++;
    }
    out->offered = offered;
    out->completed = st.completed;
    out->refused = refused;
    out->wrong_verdicts = wrong;
    out->sign_done = st.sign_done;
    out->verify_done = st.verify_done;
    out->wall_s = wall;
    out->throughput = wall > 0 ? st.completed / wall : 0;
    out->sign_throughput = wall > 0 ? st.sign_done / wall : 0;
    out->verify_throughput = wall > 0 ? st.verify_done / wall : 0;
    out->sign_p50_us = st.sign_p50_us;
    out->sign_p99_us = st.sign_p99_us;
    out->verify_p50_us = st.verify_p50_us;
    out->verify_p99_us = st.verify_p99_us;
    out->mean_batch = st.mean_batch;
    out->launch_ms_mean = st.launch_ms_mean;
    out->launch_ms_max = st.launch_ms_max;
    for (int b = 0; b < 3; b++) {
        out->sign_p50_bucket_us[b] = st.sign_p50_bucket_us[b];
        out->sign_p99_bucket_us[b] = st.sign_p99_bucket_us[b];
        out->verify_p50_bucket_us[b] = st.verify_p50_bucket_us[b];
        out->verify_p99_bucket_us[b] = st.verify_p99_bucket_us[b];
    }
    return st.completed + refused == offered ? CUSPX_OK : CUSPX_ETIMEDOUT;
}

}  // extern "C"
