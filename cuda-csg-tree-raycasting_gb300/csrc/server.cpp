// Render server (csg_server_* in include/csgrt.h): continuous batching of render
// requests over a pool of scenes kept resident under a device-memory budget.
//
// Threads.  Callers submit from any thread into a FIFO queue.  One dispatcher thread
// admits requests and makes the CUDA calls of the data path: it takes queued requests in
// arrival order while a slot (a batch in flight, one stream each) is free and their
// outputs fit in the budget, makes their scenes resident (evicting unused scenes, least
// recently used first, when the budget would be exceeded), allocates their output planes
// from a stream-ordered pool, uploads the batch's view table and launches the persistent
// view-table kernel on the slot's stream.  Requests that arrive while batches run go into
// the next free slot at once, so their work overlaps the running batches on the device:
// the persistent blocks of a later launch start as the earlier launch's blocks drain.
//
// Completion.  Requests retire one by one, not per batch: the block that renders a view's
// last tile fences its writes system-wide and stores the batch's epoch into that view's
// host-mapped flag, and a poller thread turns flags into completed requests.  An event
// recorded after each launch's last operation tells the same poller (cudaEventQuery, no
// waiting) when the whole launch is over; it then frees the slot, settles the budget and
// completes any request still open (one whose RGBA8 plane is copied to a pageable host
// buffer after the kernel).  The poller wakes every 20 us while launches are in flight,
// which answers sooner than a host function enqueued on the stream.  An RGBA8
// destination in pinned host memory is written by the kernel directly.  Requests flagged CSG_REQ_ALONE are launched one by one
// with the single-view kernel on one stream, in arrival order: the unbatched form.
//
// Budget.  Resident scenes and the output planes of admitted, unreleased requests count
// against hbm_budget.  A request whose outputs plus its scene can never fit fails with
// CSG_E_BUDGET; otherwise it waits until completions free memory.
#include <algorithm>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#if defined(__linux__)
#include <sys/prctl.h>
#endif

#include "csgrt.h"
#include "scene.hpp"
#include "scene_handle.hpp"
#include "views.hpp"

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint64_t kDefaultBudget = 40ull << 30;
constexpr int kMaxSlots = 16;
constexpr size_t kPlaneAlign = 256;
// Block shape of the server's view-table launches: per-ray stacks in local memory, the
// shape the batch autotuner picks for nearly every tree-size class of the random-tree mix
// (6% faster than shared-memory stacks on the 1,024-view batch).
#ifndef CSG_SERVER_LOCAL_STACKS
#define CSG_SERVER_LOCAL_STACKS 1
#endif
constexpr csgrt::ViewsShape kServerShape{CSG_SERVER_LOCAL_STACKS ? 4 : 8, CSG_SERVER_LOCAL_STACKS != 0};

// Size-aware scheduling (csg_server_config.order 2).  Requests fall into size levels (up
// to 2^18 rays, up to 2^20, larger), and a launch holds requests of one level only.  Each
// request gets a deadline, its arrival plus kDeadlineSlack times its rays at kNominalRate;
// the dispatcher starts with the earliest deadline whose level may launch and fills the
// launch with that level's requests, earliest deadlines first.  The largest level has one
// launch in flight at a time (its requests run in deadline order, each with the whole GPU)
// and the middle one two, so slots stay free for small requests.  A launch renders its
// views with the single-view kernel, one after another on the slot's stream, each followed
// by an event that completes its request; launches of different slots overlap on the
// device.  Launches of the smallest level (kUrgentLevels) run on a raised-priority stream,
// and no block runs long (a single-view block renders one pixel tile; the view-table
// kernel, used when CSG_SERVER_TILED_SEQUENCE is 0, gives each warp at most
// kItemsPerWarp warp tiles), so a launch of small views starts on the SMs as blocks of a
// running large one retire instead of after all of it.
constexpr double kNominalRate = 1.5e9;  // rays per second
#ifndef CSG_SERVER_DEADLINE_SLACK
#define CSG_SERVER_DEADLINE_SLACK 8.0
#endif
constexpr double kDeadlineSlack = CSG_SERVER_DEADLINE_SLACK;
#ifndef CSG_SERVER_ITEMS_PER_WARP
#define CSG_SERVER_ITEMS_PER_WARP 8
#endif
constexpr int kItemsPerWarp = CSG_SERVER_ITEMS_PER_WARP;
constexpr int kPriorityLevels = 3;
// Size-aware launches of several views as a sequence of single-view kernels (1) or one
// view-table launch (0).  Measured with the serving workload at 1,000 / 2,000 / 5,000
// req/s: the sequence delivered 1,536 / 2,584 / 2,851 Mrays/s and p99 12.6 / 46 / 153 ms,
// the view-table launches 1,536 / 2,204 / 2,151 Mrays/s and p99 19 / 71 / 257 ms.
#ifndef CSG_SERVER_TILED_SEQUENCE
#define CSG_SERVER_TILED_SEQUENCE 1
#endif
#ifndef CSG_SERVER_LARGE_IN_FLIGHT
#define CSG_SERVER_LARGE_IN_FLIGHT 1
#endif
constexpr int kLevelCap[kPriorityLevels] = {kMaxSlots, 2, CSG_SERVER_LARGE_IN_FLIGHT};
// Levels whose launches run on raised-priority streams (the smallest first).
#ifndef CSG_SERVER_URGENT_LEVELS
#define CSG_SERVER_URGENT_LEVELS 1
#endif
constexpr int kUrgentLevels = CSG_SERVER_URGENT_LEVELS;
static_assert(kUrgentLevels >= 0 && kUrgentLevels < kPriorityLevels, "urgent levels");

int size_level(const csg_request& r)
{
    const int64_t rays = (int64_t)r.w * r.h;
    return rays <= (int64_t(1) << 18) ? 0 : rays <= (int64_t(1) << 20) ? 1 : 2;
}

struct Req {
    int64_t ticket = 0;
    csg_request r{};
    double t_arrive = 0, t_launch = 0, t_done = 0;
    double deadline = 0;              // size-aware scheduling: admission order
    int status = CSG_OK;
    int batch_views = 0;
    csgrt::Planes planes{};
    void* out_mem = nullptr;          // device planes (one pool allocation)
    size_t out_bytes = 0;
    uint32_t* host_direct = nullptr;  // device address of a pinned RGBA8 destination
    cudaStream_t stream = nullptr;    // stream of the launch that renders it
    cudaEvent_t done_ev = nullptr;    // recorded after its own kernel (launches of single-view kernels)
    bool copy_back = false;           // RGBA8 copied to a pageable destination after the kernel
    bool free_enqueued = false;
    bool in_launch = false;           // a launch in flight references it
    bool released = false;            // released while in flight: deleted when the launch ends
    bool done = false;
};

struct PoolScene {
    std::string text;
    size_t bytes = 0;        // device bytes once resident
    csg_scene* dev = nullptr;
    bool uploading = false;  // bytes reserved, upload in progress
    int refs = 0;            // admitted, unfinished requests
    uint64_t last_use = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaStream_t urgent[kPriorityLevels - 1] = {};  // higher-priority streams (size-aware scheduling)
    void* dmem = nullptr;                 // counter, prefix, remaining tiles, view table
    csgrt::ViewRecord* d_views = nullptr;
    int32_t* d_prefix = nullptr;
    int32_t* d_remaining = nullptr;
    int* d_counter = nullptr;
    void* hmem = nullptr;                 // pinned staging of the same layout
    csgrt::ViewRecord* h_views = nullptr;
    int32_t* h_prefix = nullptr;
    int32_t* h_remaining = nullptr;
    unsigned int* h_flags = nullptr;      // host-mapped completion flags
    unsigned int* d_flags = nullptr;
    unsigned int epoch = 0;
    bool busy = false;
};

struct Launch {
    csg_server* srv;
    int slot;                // -1: an unbatched launch
    unsigned int epoch;
    std::vector<Req*> reqs;  // in view-table order
    cudaEvent_t done = nullptr;  // recorded after the launch's last operation
    int level = -1;          // size level of a size-aware launch
    bool flags = false;      // a view-table launch: each view stores its completion flag
};

size_t up_align(size_t v)
{
    return (v + kPlaneAlign - 1) & ~(kPlaneAlign - 1);
}

// Device bytes of a request's planes (the RGBA8 plane lives in the caller's pinned host
// buffer when there is one).
size_t plane_bytes(int planes, int64_t px, bool rgba8_on_host)
{
    size_t b = 0;
    if ((planes & CSG_PLANE_RGBA8) && !rgba8_on_host) b += up_align(px * 4);
    if (planes & CSG_PLANE_T) b += up_align(px * 4);
    if (planes & CSG_PLANE_PRIM) b += up_align(px * 4);
    if (planes & CSG_PLANE_NORMAL) b += up_align(px * 12);
    if (planes & CSG_PLANE_RGBA32F) b += up_align(px * 16);
    return b;
}

csgrt::Planes carve_planes(void* mem, int planes, int64_t px, uint32_t* rgba8_host)
{
    char* p = static_cast<char*>(mem);
    csgrt::Planes o{};
    if (planes & CSG_PLANE_RGBA8) {
        if (rgba8_host) {
            o.rgba8 = rgba8_host;
        } else {
            o.rgba8 = reinterpret_cast<uint32_t*>(p);
            p += up_align(px * 4);
        }
    }
    if (planes & CSG_PLANE_T) {
        o.t = reinterpret_cast<float*>(p);
        p += up_align(px * 4);
    }
    if (planes & CSG_PLANE_PRIM) {
        o.prim = reinterpret_cast<int32_t*>(p);
        p += up_align(px * 4);
    }
    if (planes & CSG_PLANE_NORMAL) {
        o.normal = reinterpret_cast<float*>(p);
        p += up_align(px * 12);
    }
    if (planes & CSG_PLANE_RGBA32F) o.rgba32f = reinterpret_cast<float4*>(p);
    return o;
}

}  // namespace

struct csg_server {
    csg_server_config cfg{};
    int device = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work;  // queue, slots or memory changed
    std::condition_variable cv_done;  // a request finished
    std::condition_variable cv_poll;  // a tracked launch started
    std::deque<Req*> pending;
    std::unordered_map<int64_t, Req*> reqs;
    std::vector<PoolScene> scenes;
    Slot slots[kMaxSlots];
    std::list<Launch*> tracked;       // launches in flight, watched by the poller
    std::vector<cudaEvent_t> events;  // completion events not in use
    cudaStream_t alone = nullptr;     // stream of the unbatched launches
    unsigned long long* d_capped = nullptr;  // rays of any request stopped at the iteration cap
    size_t table_head = 0;            // bytes before a slot's view records
    cudaMemPool_t pool = nullptr;
    uint64_t scene_bytes = 0, output_bytes = 0, peak = 0, use_clock = 0;
    int64_t next_ticket = 1, n_done = 0, n_batches = 0, n_evict = 0, n_rejected = 0;
    uint64_t gen = 0;                 // bumped by every event that can unblock admission
    int resident = 0, in_flight = 0;
    int level_in_flight[kPriorityLevels] = {0, 0, 0};  // size-aware launches in flight per level
    bool stop = false, stop_poll = false;
    std::thread dispatcher, poller;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    uint64_t used() const { return scene_bytes + output_bytes; }
    int free_slot() const
    {
        for (int i = 0; i < cfg.slots; ++i)
            if (!slots[i].busy) return i;
        return -1;
    }
    void complete(Req* q, double t)  // lock held
    {
        if (q->done) return;
        q->done = true;
        q->t_done = t;
        ++n_done;
    }
    void dispatch_loop();
    void poll_loop();
    bool admit(Req* q, std::vector<csg_scene*>& evicted);
    void launch(std::vector<Req*>& batch, int slot, bool alone_form);
    void finish(Launch* L, int status);
};

// End of a launch: runs on the poller once the launch's event has completed, or on the
// dispatcher when a launch could not be enqueued (no CUDA calls here).
void csg_server::finish(Launch* L, int status)
{
    {
        std::lock_guard<std::mutex> lk(mu);
        if (L->done) events.push_back(L->done);
        const double t = now();
        for (Req* q : L->reqs) {
            if (q->done_ev) {
                events.push_back(q->done_ev);
                q->done_ev = nullptr;
            }
            if (q->status == CSG_OK) q->status = status;
            complete(q, t);
            PoolScene& ps = scenes[q->r.scene];
            --ps.refs;
            ps.last_use = ++use_clock;
            q->in_launch = false;
            if (!cfg.keep_results || q->status != CSG_OK || q->released) {
                // the planes were returned to the pool on a stream, after the launch
                output_bytes -= q->out_bytes;
                q->out_bytes = 0;
                q->out_mem = nullptr;
                q->planes = csgrt::Planes{};
            }
            if (q->released) delete q;
        }
        if (L->slot >= 0) slots[L->slot].busy = false;
        if (L->level >= 0) --level_in_flight[L->level];
        --in_flight;
        ++gen;
    }
    cv_done.notify_all();
    cv_work.notify_all();
    delete L;
}

void csg_server::poll_loop()
{
#if defined(__linux__) && defined(PR_SET_TIMERSLACK)
    // This thread's sleeps between polls are 20 us; the default 50 us timer slack would
    // add up to that much to every completion.
    prctl(PR_SET_TIMERSLACK, 1000UL, 0UL, 0UL, 0UL);
#endif
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    std::vector<Launch*> watch, ended;
    std::vector<Req*> early;
    std::vector<int> ended_status;
    while (true) {
        cv_poll.wait(lk, [&] { return stop_poll || !tracked.empty(); });
        if (tracked.empty()) break;  // stop_poll
        bool any = false;
        const double t = now();
        for (Launch* L : tracked) {
            if (L->slot < 0 || !L->flags) continue;
            const volatile unsigned int* f = slots[L->slot].h_flags;
            for (size_t k = 0; k < L->reqs.size(); ++k) {
                Req* q = L->reqs[k];
                if (!q->done && !q->copy_back && f[k] == L->epoch) {
                    complete(q, t);
                    any = true;
                }
            }
        }
        if (any) cv_done.notify_all();
        // Launches end only here, so the ones in `watch` stay valid without the lock.
        watch.assign(tracked.begin(), tracked.end());
        lk.unlock();
        ended.clear();
        ended_status.clear();
        // requests rendered by their own single-view kernel end with its event
        early.clear();
        for (Launch* L : watch)
            for (Req* q : L->reqs)
                if (q->done_ev && !q->copy_back && cudaEventQuery(q->done_ev) == cudaSuccess) early.push_back(q);
        if (!early.empty()) {
            std::lock_guard<std::mutex> g(mu);
            for (Req* q : early) complete(q, t);
        }
        for (Launch* L : watch) {
            const cudaError_t e = cudaEventQuery(L->done);
            if (e == cudaErrorNotReady) continue;
            ended.push_back(L);
            ended_status.push_back(e == cudaSuccess ? CSG_OK : CSG_E_CUDA);
        }
        if (!early.empty()) cv_done.notify_all();
        if (!ended.empty()) {
            cudaGetLastError();
            {
                std::lock_guard<std::mutex> g(mu);
                for (Launch* L : ended) tracked.remove(L);
            }
            for (size_t i = 0; i < ended.size(); ++i) finish(ended[i], ended_status[i]);
        } else {
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
        lk.lock();
    }
}

// Admission of the queue head (lock held): reserves its outputs and makes room for its
// scene.  Returns false if it must wait; a request that can never fit is failed.
bool csg_server::admit(Req* q, std::vector<csg_scene*>& evicted)
{
    PoolScene& ps = scenes[q->r.scene];
    const bool have = ps.dev || ps.uploading;
    const uint64_t need = q->out_bytes + (have ? 0 : ps.bytes);
    if (need > cfg.hbm_budget) {
        q->status = CSG_E_BUDGET;
        return true;
    }
    if (used() + need > cfg.hbm_budget) {
        // evict only if that makes enough room
        uint64_t freeable = 0;
        for (int i = 0; i < (int)scenes.size(); ++i)
            if (scenes[i].dev && scenes[i].refs == 0 && i != q->r.scene) freeable += scenes[i].bytes;
        if (used() - freeable + need > cfg.hbm_budget) return false;  // wait for memory
        while (used() + need > cfg.hbm_budget) {
            int victim = -1;  // least recently used resident scene no admitted request holds
            for (int i = 0; i < (int)scenes.size(); ++i) {
                const PoolScene& c = scenes[i];
                if (c.dev && c.refs == 0 && i != q->r.scene &&
                    (victim < 0 || c.last_use < scenes[victim].last_use))
                    victim = i;
            }
            evicted.push_back(scenes[victim].dev);
            scenes[victim].dev = nullptr;
            scene_bytes -= scenes[victim].bytes;
            --resident;
            ++n_evict;
        }
    }
    output_bytes += q->out_bytes;
    if (!have) {
        scene_bytes += ps.bytes;  // reserved now, uploaded by the dispatcher
        ps.uploading = true;
    }
    peak = std::max(peak, used());
    ++ps.refs;
    q->in_launch = true;
    return true;
}

// Enqueues one launch (lock not held): uploads, output planes, the kernel, the copies to
// pageable host buffers, the frees and the completion host function.
void csg_server::launch(std::vector<Req*>& batch, int slot, bool alone_form)
{
    // scenes to upload (reserved in admit)
    std::vector<int> uploads;
    std::vector<std::string> texts;
    {
        std::lock_guard<std::mutex> g(mu);
        for (Req* q : batch)
            if (!scenes[q->r.scene].dev &&
                std::find(uploads.begin(), uploads.end(), q->r.scene) == uploads.end()) {
                uploads.push_back(q->r.scene);
                texts.push_back(scenes[q->r.scene].text);
            }
    }
    std::vector<csg_scene*> made(uploads.size(), nullptr);
    int rc = CSG_OK;
    for (size_t i = 0; i < uploads.size(); ++i) {
        const int r = csg_scene_create(texts[i].data(), texts[i].size(), &made[i], nullptr, 0);
        if (r != CSG_OK) rc = r;
    }
    std::vector<const csg_scene*> sc(batch.size(), nullptr);
    {
        std::lock_guard<std::mutex> g(mu);
        for (size_t i = 0; i < uploads.size(); ++i) {
            PoolScene& ps = scenes[uploads[i]];
            ps.uploading = false;
            if (made[i]) {
                ps.dev = made[i];
                ++resident;
            } else {
                scene_bytes -= ps.bytes;
            }
        }
        for (size_t i = 0; i < batch.size(); ++i) sc[i] = scenes[batch[i]->r.scene].dev;
    }
    if (cfg.order == 2 && batch.size() > 1) {
        // earliest deadline first in the view table too
        std::stable_sort(batch.begin(), batch.end(), [](const Req* a, const Req* b) { return a->deadline < b->deadline; });
        for (size_t i = 0; i < batch.size(); ++i) sc[i] = scenes[batch[i]->r.scene].dev;
    }
    if (cfg.order == 1 && batch.size() > 1) {
        // longest first: the launch's tail is short, at the cost of later completions for
        // the cheap views
        std::vector<size_t> idx(batch.size());
        for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
        auto cost = [&](size_t i) {
            const Req* q = batch[i];
            return (double)q->r.w * q->r.h * (1.0 + (sc[i] ? sc[i]->dev.n_prims : 0));
        };
        std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return cost(a) > cost(b); });
        std::vector<Req*> b2(batch.size());
        std::vector<const csg_scene*> s2(batch.size());
        for (size_t i = 0; i < idx.size(); ++i) {
            b2[i] = batch[idx[i]];
            s2[i] = sc[idx[i]];
        }
        batch.swap(b2);
        sc.swap(s2);
    }
    cudaStream_t st = alone_form ? alone : slots[slot].stream;
    int level = -1;
    if (!alone_form && cfg.order == 2) {
        level = 0;
        for (const Req* q : batch) level = std::max(level, size_level(q->r));
        if (level < kUrgentLevels && slots[slot].urgent[level]) st = slots[slot].urgent[level];
    }
    Launch* L = new Launch{this, slot, 0u, batch};
    L->level = level;
    const int tw = cfg.warp_tile_w;
    cudaError_t e = cudaSuccess;
    if (rc == CSG_OK) {
        const double tl = now();
        for (Req* q : batch) {
            q->t_launch = tl;
            q->stream = st;
            q->batch_views = (int)batch.size();
            if (q->out_bytes) {
                e = cudaMallocFromPoolAsync(&q->out_mem, q->out_bytes, pool, st);
                if (e != cudaSuccess) break;
            }
            q->planes = carve_planes(q->out_mem, cfg.planes, (int64_t)q->r.w * q->r.h, q->host_direct);
        }
    }
    if (rc == CSG_OK && e == cudaSuccess) {
        if (!alone_form && cfg.order == 2 && (batch.size() == 1 || CSG_SERVER_TILED_SEQUENCE)) {
            // size-aware launch of single-view kernels, one per view in deadline order, each
            // followed by an event that completes its request
            for (size_t k = 0; k < batch.size() && e == cudaSuccess; ++k) {
                Req* q = batch[k];
                csgrt::Camera cam;
                std::memcpy(cam.v, &q->r.cam, sizeof(cam.v));
                e = csgrt::launch_render(sc[k]->dev, sc[k]->center, cam, q->r.light_dir, q->r.w, q->r.h, q->planes,
                                         d_capped, st);
                if (e == cudaSuccess && !q->copy_back) {
                    {
                        std::lock_guard<std::mutex> g(mu);
                        if (!events.empty()) {
                            q->done_ev = events.back();
                            events.pop_back();
                        }
                    }
                    if (!q->done_ev) e = cudaEventCreateWithFlags(&q->done_ev, cudaEventDisableTiming);
                    if (e == cudaSuccess) e = cudaEventRecord(q->done_ev, st);
                }
            }
        } else if (alone_form) {
            // the unbatched form: the single-view kernel; the launch's event completes it
            Req* q = batch[0];
            csgrt::Camera cam;
            std::memcpy(cam.v, &q->r.cam, sizeof(cam.v));
            e = csgrt::launch_render(sc[0]->dev, sc[0]->center, cam, q->r.light_dir, q->r.w, q->r.h, q->planes,
                                     d_capped, st);
        } else {
            // view table in arrival order, tile prefix, per-view remaining tiles
            Slot& S = slots[slot];
            L->epoch = ++S.epoch;
            L->flags = true;
            int32_t sd = 4, live = 1;
            bool rolled = false;
            int64_t total = 0;
            for (size_t k = 0; k < batch.size(); ++k) {
                const Req* q = batch[k];
                csgrt::make_view_record(sc[k]->dev, d_capped, reinterpret_cast<const float*>(&q->r.cam),
                                        q->r.light_dir, q->r.w, q->r.h, q->planes, tw, S.h_views[k]);
                S.h_views[k].host_out = q->host_direct ? 1 : 0;
                const int64_t tiles = csgrt::view_tiles(q->r.w, q->r.h, tw);
                S.h_prefix[k] = (int32_t)total;
                S.h_remaining[k] = (int32_t)tiles;
                total += tiles;
                sd = std::max(sd, sc[k]->dev.stack_class);
                live = std::max(live, sc[k]->dev.live_words);
                rolled = rolled || sc[k]->dev.rolled;
            }
            const size_t nv = batch.size();
            S.h_prefix[nv] = (int32_t)total;
            // counter (0), prefix, remaining and the batch's view records in one copy
            e = cudaMemcpyAsync(S.dmem, S.hmem, table_head + nv * sizeof(csgrt::ViewRecord), cudaMemcpyHostToDevice,
                                st);
            if (e == cudaSuccess) {
                csgrt::ViewsLaunch vl;
                vl.views = S.d_views;
                vl.prefix = S.d_prefix;
                vl.counter = S.d_counter;
                vl.n_views = (int32_t)nv;
                vl.n_items = (int32_t)total;
                vl.tw_log2 = csgrt::tile_log2(tw);
                vl.live_words = live;
                vl.iter_cap = csgrt::iteration_cap();
                vl.remaining = S.d_remaining;
                vl.done_flags = S.d_flags;
                vl.epoch = L->epoch;
                vl.items_per_warp = cfg.order == 2 ? kItemsPerWarp : 0;  // (level >= 0)
                e = csgrt::launch_views(vl, csgrt::stack_class_for_depth(sd), rolled, kServerShape, device, st);
            }
        }
        for (Req* q : batch) {
            if (e != cudaSuccess) break;
            if (q->copy_back && q->planes.rgba8)
                e = cudaMemcpyAsync(q->r.host_rgba8, q->planes.rgba8, (size_t)q->r.w * q->r.h * 4,
                                    cudaMemcpyDeviceToHost, st);
        }
    }
    if (rc == CSG_OK && e == cudaSuccess && !cfg.keep_results)
        for (Req* q : batch) {
            if (!q->out_mem || e != cudaSuccess) continue;
            e = cudaFreeAsync(q->out_mem, st);
            q->free_enqueued = e == cudaSuccess;
        }
    if (rc == CSG_OK && e == cudaSuccess) {
        {
            std::lock_guard<std::mutex> g(mu);
            if (!events.empty()) {
                L->done = events.back();
                events.pop_back();
            }
        }
        if (!L->done) e = cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(L->done, st);
        if (e == cudaSuccess) {
            {
                std::lock_guard<std::mutex> g(mu);
                tracked.push_back(L);
            }
            cv_poll.notify_one();
        }
    }
    if (rc != CSG_OK || e != cudaSuccess) {
        // nothing more is enqueued for this launch: return its planes and fail it
        cudaStreamSynchronize(st);
        for (Req* q : batch)
            if (q->out_mem && !q->free_enqueued) {
                cudaFreeAsync(q->out_mem, st);
                q->free_enqueued = true;
            }
        cudaStreamSynchronize(st);
        finish(L, rc != CSG_OK ? rc : CSG_E_CUDA);
    }
}

void csg_server::dispatch_loop()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        cv_work.wait(lk, [&] {
            if (pending.empty()) return stop;
            if (pending.front()->r.flags & CSG_REQ_ALONE) return true;
            return free_slot() >= 0;
        });
        if (pending.empty() && stop) break;

        // Size-aware scheduling: the queue in deadline order (stable: equal deadlines keep
        // their arrival order).
        if (cfg.order == 2 && pending.size() > 1)
            std::stable_sort(pending.begin(), pending.end(),
                             [](const Req* a, const Req* b) { return a->deadline < b->deadline; });
        // Form the next launch: one unbatched request, or a batch for a free slot.
        std::vector<Req*> batch;
        std::vector<csg_scene*> evicted;
        const bool alone_form = (pending.front()->r.flags & CSG_REQ_ALONE) != 0;
        const int slot = alone_form ? -1 : free_slot();
        bool blocked = false, rejected = false;
        // size-aware: the level of the earliest deadline that may launch (-1: none may)
        int level = -1;
        if (cfg.order == 2 && !alone_form) {
            for (const Req* q : pending) {
                if (q->r.flags & CSG_REQ_ALONE) break;
                const int l = size_level(q->r);
                if (level_in_flight[l] < kLevelCap[l]) {
                    level = l;
                    break;
                }
            }
            if (level < 0) {
                // every level with queued requests is at its cap: wait for a launch to end
                const uint64_t g = gen;
                cv_work.wait(lk, [&] { return gen != g || stop; });
                continue;
            }
        }
        for (auto it = pending.begin(); it != pending.end() && (int)batch.size() < (alone_form ? 1 : cfg.max_batch_views);) {
            Req* q = *it;
            if (((q->r.flags & CSG_REQ_ALONE) != 0) != alone_form) break;
            if (level >= 0 && size_level(q->r) != level) {
                ++it;
                continue;
            }
            if (!admit(q, evicted)) {
                blocked = true;
                break;
            }
            it = pending.erase(it);
            if (q->status != CSG_OK) {
                complete(q, now());
                ++n_rejected;
                rejected = true;
                continue;
            }
            batch.push_back(q);
        }
        if (rejected) cv_done.notify_all();
        if (batch.empty()) {
            if (blocked) {
                // nothing admissible until a launch finishes or a result is released
                const uint64_t g = gen;
                lk.unlock();
                for (csg_scene* s : evicted) csg_scene_destroy(s);
                lk.lock();
                if (stop && in_flight == 0 && gen == g) {
                    // shutting down with requests that no release will ever make room for
                    for (Req* q : pending) {
                        q->status = CSG_E_BUDGET;
                        complete(q, now());
                        ++n_rejected;
                    }
                    pending.clear();
                    cv_done.notify_all();
                    continue;
                }
                cv_work.wait(lk, [&] { return gen != g || (stop && in_flight == 0); });
            }
            continue;
        }
        if (slot >= 0) slots[slot].busy = true;
        if (level >= 0) ++level_in_flight[level];
        ++in_flight;
        ++n_batches;
        lk.unlock();
        for (csg_scene* s : evicted) csg_scene_destroy(s);
        launch(batch, slot, alone_form);
        lk.lock();
    }
}

extern "C" {

int csg_server_create(const csg_server_config* cfg_in, csg_server** out)
{
    if (!out) return CSG_E_ARG;
    *out = nullptr;
    csg_server_config cfg{};
    if (cfg_in) cfg = *cfg_in;
    if (cfg.hbm_budget == 0) cfg.hbm_budget = kDefaultBudget;
    if (cfg.slots == 0) cfg.slots = 4;
    if (cfg.max_batch_views == 0) cfg.max_batch_views = 256;
    if (cfg.warp_tile_w == 0) cfg.warp_tile_w = 8;
    if (cfg.planes == 0) cfg.planes = CSG_PLANE_RGBA8;
    if (cfg.slots < 1 || cfg.slots > kMaxSlots || cfg.max_batch_views < 1 || cfg.max_batch_views > 4096 ||
        (cfg.warp_tile_w != 4 && cfg.warp_tile_w != 8 && cfg.warp_tile_w != 16 && cfg.warp_tile_w != 32) ||
        (cfg.planes & ~31) != 0 || cfg.order < 0 || cfg.order > 2)
        return CSG_E_ARG;
    csg_server* s = new (std::nothrow) csg_server();
    if (!s) return CSG_E_CUDA;
    s->cfg = cfg;
    s->t0 = Clock::now();
    cudaError_t e = cudaGetDevice(&s->device);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    if (e == cudaSuccess) e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = UINT64_MAX;  // keep freed blocks for reuse instead of returning them
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->alone, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_capped, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(s->d_capped, 0, sizeof(unsigned long long));
    const size_t nv = (size_t)cfg.max_batch_views;
    // [counter | pad to 16][prefix: nv + 1][remaining: nv][pad to 16][views], the same
    // layout staged on the host, so that one copy (its length set by the views in the
    // batch) resets the counter and carries the whole table
    const size_t head = (16 + (2 * nv + 1) * sizeof(int32_t) + 15) & ~size_t(15);
    const size_t dbytes = head + nv * sizeof(csgrt::ViewRecord);
    s->table_head = head;
    for (int i = 0; i < cfg.slots && e == cudaSuccess; ++i) {
        Slot& S = s->slots[i];
        e = cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess && cfg.order == 2) {
            // higher priorities for launches of smaller views (numerically lower is higher)
            int least = 0, greatest = 0;
            e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
            for (int k = 0; k < kPriorityLevels - 1 && e == cudaSuccess; ++k) {
                const int prio = greatest + (least - greatest) * k / (kPriorityLevels - 1);
                e = cudaStreamCreateWithPriority(&S.urgent[k], cudaStreamNonBlocking, prio);
            }
        }
        if (e == cudaSuccess) e = cudaMalloc(&S.dmem, dbytes);
        if (e == cudaSuccess) e = cudaMallocHost(&S.hmem, dbytes);
        if (e == cudaSuccess)
            e = cudaHostAlloc(reinterpret_cast<void**>(&S.h_flags), nv * sizeof(unsigned int), cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&S.d_flags), S.h_flags, 0);
        if (e != cudaSuccess) break;
        std::memset(S.h_flags, 0, nv * sizeof(unsigned int));
        std::memset(S.hmem, 0, head);  // the staged counter stays 0
        S.d_counter = static_cast<int*>(S.dmem);
        S.d_prefix = reinterpret_cast<int32_t*>(static_cast<char*>(S.dmem) + 16);
        S.d_remaining = S.d_prefix + nv + 1;
        S.d_views = reinterpret_cast<csgrt::ViewRecord*>(static_cast<char*>(S.dmem) + head);
        S.h_prefix = reinterpret_cast<int32_t*>(static_cast<char*>(S.hmem) + 16);
        S.h_remaining = S.h_prefix + nv + 1;
        S.h_views = reinterpret_cast<csgrt::ViewRecord*>(static_cast<char*>(S.hmem) + head);
    }
    if (e != cudaSuccess) {
        csg_server_destroy(s);
        return CSG_E_CUDA;
    }
    s->dispatcher = std::thread([s] { s->dispatch_loop(); });
    s->poller = std::thread([s] { s->poll_loop(); });
    *out = s;
    return CSG_OK;
}

int csg_server_destroy(csg_server* s)
{
    if (!s) return CSG_E_ARG;
    if (s->dispatcher.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        s->dispatcher.join();
    }
    // wait for every launch (the poller finishes them)
    {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_done.wait(lk, [&] { return s->in_flight == 0; });
        s->stop_poll = true;
    }
    s->cv_poll.notify_all();
    if (s->poller.joinable()) s->poller.join();
    for (int i = 0; i < kMaxSlots; ++i) {
        if (s->slots[i].stream) cudaStreamSynchronize(s->slots[i].stream);
        for (cudaStream_t u : s->slots[i].urgent)
            if (u) cudaStreamSynchronize(u);
    }
    if (s->alone) cudaStreamSynchronize(s->alone);
    for (auto& kv : s->reqs) {
        if (kv.second->out_mem && !kv.second->free_enqueued) cudaFreeAsync(kv.second->out_mem, s->alone);
        delete kv.second;
    }
    if (s->alone) cudaStreamSynchronize(s->alone);
    for (PoolScene& p : s->scenes)
        if (p.dev) csg_scene_destroy(p.dev);
    for (int i = 0; i < kMaxSlots; ++i) {
        Slot& S = s->slots[i];
        if (S.stream) cudaStreamDestroy(S.stream);
        for (cudaStream_t u : S.urgent)
            if (u) cudaStreamDestroy(u);
        if (S.dmem) cudaFree(S.dmem);
        if (S.hmem) cudaFreeHost(S.hmem);
        if (S.h_flags) cudaFreeHost(S.h_flags);
    }
    if (s->alone) cudaStreamDestroy(s->alone);
    for (cudaEvent_t ev : s->events) cudaEventDestroy(ev);
    if (s->d_capped) cudaFree(s->d_capped);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return CSG_OK;
}

int csg_server_add_scene(csg_server* s, const char* text, size_t len, int32_t* id, char* err, size_t errlen)
{
    if (!s || !id || (!text && len)) return CSG_E_ARG;
    csgrt::HostTree tree;
    std::string msg;
    const int rc = csgrt::parse_tree(std::string_view(text ? text : "", len), tree, msg);
    if (rc != csgrt::kOk) {
        if (err && errlen) {
            const size_t n = std::min(errlen - 1, msg.size());
            std::memcpy(err, msg.data(), n);
            err[n] = '\0';
        }
        return rc;
    }
    csgrt::PackedScene pk;
    csgrt::pack_scene(tree, pk);
    PoolScene ps;
    ps.text.assign(text ? text : "", len);
    ps.bytes = csgrt::scene_layout(tree.nodes.size(), tree.prims.size(), pk.kids.size(), pk.bvh.size()).total;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->scenes.size() >= (size_t)INT_MAX) return CSG_E_CAPACITY;
    *id = (int32_t)s->scenes.size();
    s->scenes.push_back(std::move(ps));
    return CSG_OK;
}

int csg_server_preload(csg_server* s, int32_t id)
{
    if (!s) return CSG_E_ARG;
    std::string text;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (id < 0 || id >= (int32_t)s->scenes.size()) return CSG_E_ARG;
        PoolScene& ps = s->scenes[id];
        if (ps.dev || ps.uploading) return CSG_OK;
        if (s->used() + ps.bytes > s->cfg.hbm_budget) return CSG_E_BUDGET;
        text = ps.text;
        s->scene_bytes += ps.bytes;  // reserved
        ps.uploading = true;
        ++ps.refs;
    }
    csg_scene* made = nullptr;
    const int rc = csg_scene_create(text.data(), text.size(), &made, nullptr, 0);
    std::lock_guard<std::mutex> lk(s->mu);
    PoolScene& ps = s->scenes[id];
    --ps.refs;
    ps.uploading = false;
    ++s->gen;
    if (rc != CSG_OK) {
        s->scene_bytes -= ps.bytes;
        return rc;
    }
    ps.dev = made;
    ps.last_use = ++s->use_clock;
    ++s->resident;
    s->peak = std::max(s->peak, s->used());
    return CSG_OK;
}

static int submit_at(csg_server* s, const csg_request* r, double t_arrive, int64_t* ticket)
{
    if (!s || !r || !ticket) return CSG_E_ARG;
    if (r->w <= 0 || r->h <= 0 || (int64_t)r->w * r->h > (1ll << 28)) return CSG_E_ARG;
    Req* q = new (std::nothrow) Req();
    if (!q) return CSG_E_CUDA;
    q->r = *r;
    if (r->host_rgba8 && (s->cfg.planes & CSG_PLANE_RGBA8)) {
        // pinned (page-locked, device-mapped) destinations are written by the kernel itself
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, r->host_rgba8) == cudaSuccess && a.type == cudaMemoryTypeHost &&
            a.devicePointer)
            q->host_direct = static_cast<uint32_t*>(a.devicePointer);
        else
            q->copy_back = true;
        cudaGetLastError();
    }
    q->out_bytes = plane_bytes(s->cfg.planes, (int64_t)r->w * r->h, q->host_direct != nullptr);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (r->scene < 0 || r->scene >= (int32_t)s->scenes.size() || s->stop) {
            delete q;
            return CSG_E_ARG;
        }
        q->ticket = s->next_ticket++;
        q->t_arrive = t_arrive < 0 ? s->now() : t_arrive;
        // (unbatched requests keep their arrival order: they are the plain form)
        q->deadline = q->t_arrive + ((r->flags & CSG_REQ_ALONE) ? 0.0 : kDeadlineSlack * (double)r->w * r->h / kNominalRate);
        s->reqs[q->ticket] = q;
        s->pending.push_back(q);
        ++s->gen;
        *ticket = q->ticket;
    }
    s->cv_work.notify_all();
    return CSG_OK;
}

int csg_server_submit(csg_server* s, const csg_request* r, int64_t* ticket)
{
    return submit_at(s, r, -1.0, ticket);
}

int csg_server_wait(csg_server* s, int64_t ticket, double timeout_s, csg_result* out)
{
    if (!s) return CSG_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return CSG_E_ARG;
    Req* q = it->second;
    if (timeout_s < 0) {
        s->cv_done.wait(lk, [&] { return q->done; });
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return q->done; })) {
        return CSG_E_TIMEOUT;
    }
    if (out) {
        out->status = q->status;
        out->batch_views = q->batch_views;
        out->t_arrive = q->t_arrive;
        out->t_launch = q->t_launch;
        out->t_done = q->t_done;
        out->planes = csg_planes{q->planes.rgba8, reinterpret_cast<float*>(q->planes.rgba32f), q->planes.t,
                                 q->planes.prim, q->planes.normal};
    }
    return CSG_OK;
}

int csg_server_release(csg_server* s, int64_t ticket)
{
    if (!s) return CSG_E_ARG;
    void* mem = nullptr;
    cudaStream_t st = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end() || !it->second->done) return CSG_E_ARG;
        Req* q = it->second;
        s->reqs.erase(it);
        if (q->in_launch) {
            // its launch still runs (the request retired early): the launch's end settles
            // the budget and deletes it; its planes go back to the pool after that launch
            q->released = true;
            if (q->out_mem && !q->free_enqueued) {
                mem = q->out_mem;
                q->free_enqueued = true;
                st = q->stream;  // ordered after the launch on its own stream
            }
        } else {
            mem = q->free_enqueued ? nullptr : q->out_mem;
            st = s->alone;
            s->output_bytes -= q->out_bytes;
            delete q;
            ++s->gen;
        }
    }
    int rc = CSG_OK;
    if (mem) {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(s->device);
        if (cudaFreeAsync(mem, st) != cudaSuccess) rc = CSG_E_CUDA;
        cudaSetDevice(prev);
    }
    s->cv_work.notify_all();
    return rc;
}

int csg_server_replay(csg_server* s, const csg_request* reqs, const double* arrival_s, int32_t n,
                      csg_result* results, int64_t* tickets, double* wall_s)
{
    if (!s || !reqs || !arrival_s || n <= 0) return CSG_E_ARG;
    for (int32_t i = 1; i < n; ++i)
        if (arrival_s[i] < arrival_s[i - 1]) return CSG_E_ARG;
    std::vector<int64_t> tk(n, 0);
    const double start = s->now();
    int rc = CSG_OK;
    for (int32_t i = 0; i < n && rc == CSG_OK; ++i) {
        const double target = start + arrival_s[i];
        while (true) {
            const double left = target - s->now();
            if (left <= 0) break;
            if (left > 300e-6) std::this_thread::sleep_for(std::chrono::duration<double>(left - 200e-6));
        }
        rc = submit_at(s, &reqs[i], target, &tk[i]);
    }
    double last = start;
    for (int32_t i = 0; i < n; ++i) {
        if (!tk[i]) continue;
        csg_result r{};
        csg_server_wait(s, tk[i], -1.0, &r);
        last = std::max(last, r.t_done);
        if (results) results[i] = r;
        if (tickets) tickets[i] = tk[i];
        else csg_server_release(s, tk[i]);
    }
    if (wall_s) *wall_s = last - start;
    return rc;
}

int csg_server_stats_get(csg_server* s, csg_server_stats* o)
{
    if (!s || !o) return CSG_E_ARG;
    // rays stopped at the iteration cap so far (a count that only grows; launches still in
    // flight may add to it)
    unsigned long long capped = 0;
    if (cudaMemcpy(&capped, s->d_capped, sizeof(capped), cudaMemcpyDeviceToHost) != cudaSuccess) return CSG_E_CUDA;
    o->capped_rays = capped;
    std::lock_guard<std::mutex> lk(s->mu);
    o->budget = s->cfg.hbm_budget;
    o->scene_bytes = s->scene_bytes;
    o->output_bytes = s->output_bytes;
    o->peak_bytes = s->peak;
    o->requests_done = s->n_done;
    o->batches = s->n_batches;
    o->evictions = s->n_evict;
    o->rejected = s->n_rejected;
    o->scenes = (int32_t)s->scenes.size();
    o->resident_scenes = s->resident;
    int busy = 0;
    for (int i = 0; i < s->cfg.slots; ++i) busy += s->slots[i].busy ? 1 : 0;
    o->slots_busy = busy;
    o->pending = (int32_t)s->pending.size();
    return CSG_OK;
}

double csg_server_clock(const csg_server* s)
{
    return s ? s->now() : 0.0;
}

}  // extern "C"
