// pa_batch.cu -- many blocks on one GPU: a pool of slots (one CUDA stream + working set each), the
// static-seed spectrum cache, batched runs (optionally one CUDA graph per batch, or one persistent lane
// launch, pa_lanes.cuh), served blocks (pa_submit / pa_poll, admission by free slot and HBM budget) and
// the three-pass split autotuner.
//
// The reference has none of this (one block at a time, PrivacyAmplification.cu:1686-2118); the
// per-block work is the same key-block / seed-spectrum kernels the single-block engine runs.
#include "pa_engine_impl.h"
#include "pa_lanes.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <new>
#include <numeric>
#include <unordered_map>
#include <vector>

using pa::BlockGeom;

namespace pa_host {

namespace {

constexpr int kFp32MaxLogNp = 27;  // the FP32 path serves n <= 2^27

struct Mirror {  // pinned host copy of a served block's statistics
    unsigned long long cnt[2];
    unsigned int resid;
    int err;
};

struct SeedEntry {
    BlockGeom g{};
    float2* spec = nullptr;          // FP32 spectrum in the key path's layout
    uint32_t* seed = nullptr;        // seed words (for the exact recompute)
    unsigned long long* cnt = nullptr;  // popcount of the placed seed
    size_t bytes = 0;
    bool live = false;
};

// Grouped launches (pa_group.cu): jobs of one geometry, at least min_group of them (pa_set_groups), run
// as one launch per pass for up to 2^group_log_bits bits of cyclic length per group; larger blocks run
// alone.  Groups of a geometry spread over the batch's slot streams like single blocks, so passes of
// different groups overlap.
constexpr uint32_t kMinGroup = 4;
constexpr int kGroupLogBits = 24;  // measured best for 2^27-bit banks of 2^18 .. 2^22-bit blocks

// A group's working set: Y, Z and the group's own seed spectra (complex values each), bit rows / planes.
struct GroupBuf {
    float2* work = nullptr;
    float2* work2 = nullptr;
    float2* spec = nullptr;
    uint32_t* planes = nullptr;
    size_t work_cap = 0, planes_cap = 0, bytes = 0;
};

// One group of a batch: `count` jobs of geometry g, their entries from entry_off of the batch's table,
// its working set the pool's group buffer of the same index.
struct GroupChunk {
    BlockGeom g{};
    uint32_t flags = 0;
    bool dynamic = false;  // every job brings its own seed
    uint32_t count = 0;
    size_t entry_off = 0;
    double cost = 0.0;
    pa::PassMaps maps{};
    std::vector<int> jobs;  // job indices, in entry order
};

size_t group_planes_stride(const BlockGeom& g) { return (size_t(1) << g.log_np) / 32 + 64; }

}  // namespace

struct Slot {
    int cap = 0;  // log2 of the largest cyclic length the buffers hold
    size_t bytes = 0;
    cudaStream_t s = nullptr;
    float2* work = nullptr;   // pass A output / exact-path residues
    float2* work2 = nullptr;  // pass B output / exact-path scratch
    float2* spec = nullptr;   // dynamic seed spectrum / exact seed transform
    uint32_t* planes = nullptr;
    int* err = nullptr;
    unsigned long long* cnt = nullptr;  // served block: [0] key, [1] seed popcount
    unsigned int* resid = nullptr;
    uint32_t *seed = nullptr, *ks = nullptr, *kr = nullptr, *out = nullptr;  // served-block staging
    Mirror* host = nullptr;
    pa::PassMaps maps{};
    int maps_key = -1;
    pa::NttTables* ntt = nullptr;
    cudaEvent_t done = nullptr, join = nullptr;
    // served block in flight
    bool busy = false;
    uint64_t ticket = 0;
    pa_job job{};
    BlockGeom g{};
    int seed_id = -1;
    uint64_t last_use = 0;
};

// A static seed's spectrum in the lane layout (pa_lanes.cuh).
struct LaneSpec {
    float2* spec = nullptr;
    unsigned long long* cnt = nullptr;  // [0] unused, [1] popcount of the placed seed, then a scratch word
    size_t bytes = 0;
};

// A captured persistent launch and the job array it reads.
struct LaneGraph {
    cudaGraphExec_t exec = nullptr;
    pa::LaneJob* jobs = nullptr;
};

// The persistent lane engine's working sets: `lanes` lanes of T CTAs, each with a block's arrays for
// cyclic lengths up to 2^cap.
struct LaneSet {
    int T = 0, lanes = 0, cap = 0;
    size_t bytes = 0, smem = 0;
    float2 *work = nullptr, *work2 = nullptr, *spec = nullptr;
    uint32_t* planes = nullptr;
    size_t work_stride = 0, planes_stride = 0;
    CUtensorMap* maps = nullptr;   // [lane][log_n1][Y, Z]
    unsigned int* ctl = nullptr;   // next, bar[lanes], slot[lanes], err[lanes]
    pa::LaneJob* jobs = nullptr;   // uncaptured launches
    uint32_t job_cap = 0;
    int early_b[pa::kLaneMaps] = {}, early_c[pa::kLaneMaps] = {};
    std::map<std::array<uint64_t, 4>, LaneSpec> spectra;
    std::unordered_map<uint64_t, LaneGraph> graphs;
};

// The device-resident serving loop (pa_serve_*): the lane kernel in serving mode, fed from a ring of
// request slots in pinned host memory.
struct ServeLoop {
    pa::ServeSlot* ring = nullptr;  // pinned host memory
    pa::ServeCtl* ctl = nullptr;    // pinned host memory
    pa::ServeSlot* d_ring = nullptr;  // the same memory as the device addresses it
    pa::ServeCtl* d_ctl = nullptr;
    uint32_t size = 0;
    unsigned long long* claimed = nullptr;  // device
    pa::LaneJob* lane_job = nullptr;        // device
    unsigned long long* lane_stats = nullptr;
    uint32_t* stage = nullptr;  // device: per lane, a request's inputs copied from host memory
    size_t stage_stride = 0;
    cudaStream_t s = nullptr;
    cudaEvent_t ended = nullptr;  // recorded after each launch of the loop
    bool launched = false;
    bool failed = false;  // a launch of the loop ended with a lane error or a request it took unfinished
    uint64_t next_ticket = 0;
    std::vector<uint64_t> owner;  // per ring slot: the ticket in it, or ~0 when free
    std::vector<pa_job> jobs;     // per ring slot: the request as submitted (exact recompute)
    std::vector<BlockGeom> geoms;
    unsigned long long idle_ns = 2000000000ull;  // the loop ends after two seconds without requests
};

struct Pool {
    std::vector<Slot*> slots;
    std::vector<SeedEntry> seeds;
    uint64_t budget = 0;
    size_t used = 0;
    int max_slots = 16;
    int batch_slots = 8;
    uint64_t clock = 0;
    uint64_t next_ticket = 1;
    // batch state
    cudaEvent_t fork = nullptr, b0 = nullptr, b1 = nullptr;
    unsigned long long* job_cnt = nullptr;  // [count][2]
    unsigned int* job_resid = nullptr;      // [count]
    uint32_t job_cap = 0;
    std::vector<pa_job> jobs;
    std::vector<BlockGeom> geoms;
    cudaStream_t batch_stream = nullptr;
    bool batch_pending = false;
    std::unordered_map<uint64_t, cudaGraphExec_t> graphs;
    // grouped launches: working sets, the pending batch's groups and their entry table (a captured
    // graph keeps a table of its own, freed with it)
    std::vector<GroupBuf> gbufs;
    std::vector<GroupChunk> chunks;
    std::vector<pa::GroupEntry> hentries;
    pa::GroupEntry* gentries = nullptr;
    size_t gentries_cap = 0;
    std::unordered_map<uint64_t, pa::GroupEntry*> graph_entries;
    uint32_t min_group = kMinGroup;
    int group_log_bits = kGroupLogBits;
    // persistent lane launches
    LaneSet* lanes = nullptr;
    int lane_ctas = 4;        // CTAs per lane (pa_set_lanes)
    int lane_cap = 0;         // log2 of the cyclic length the lanes are sized for (0: the batch's largest)
    bool batch_lanes = false; // the pending batch ran on the lanes
    ServeLoop* serve = nullptr;
};

namespace {

void free_slot(Pool* p, Slot* sl) {
    if (!sl) return;
    if (sl->s) cudaStreamSynchronize(sl->s);
    cudaFree(sl->work);
    cudaFree(sl->work2);
    cudaFree(sl->spec);
    cudaFree(sl->planes);
    cudaFree(sl->err);
    cudaFree(sl->cnt);
    cudaFree(sl->resid);
    cudaFree(sl->seed);
    cudaFree(sl->ks);
    cudaFree(sl->kr);
    cudaFree(sl->out);
    cudaFreeHost(sl->host);
    pa::free_ntt_tables(sl->ntt);
    if (sl->done) cudaEventDestroy(sl->done);
    if (sl->join) cudaEventDestroy(sl->join);
    if (sl->s) cudaStreamDestroy(sl->s);
    p->used -= std::min(p->used, sl->bytes);
    delete sl;
}

size_t slot_bytes(int cap) {
    const size_t np = size_t(1) << cap;
    const size_t np32 = std::min(np, size_t(1) << kFp32MaxLogNp);
    return 3 * (np / 2) * sizeof(float2) - (np - np32) / 2 * sizeof(float2) + 5 * (np / 8 + 256);
}

int new_slot(pa_engine* e, Pool* p, int cap, Slot** out) {
    Slot* sl = new (std::nothrow) Slot();
    if (!sl) return PA_ERR_INVALID_ARG;
    sl->cap = cap;
    const size_t np = size_t(1) << cap;
    const size_t np32 = std::min(np, size_t(1) << kFp32MaxLogNp);
    const size_t words = np / 32 + 64;
    cudaError_t err = cudaSuccess;
    auto A = [&](void** ptr, size_t bytes) {
        if (err == cudaSuccess) err = cudaMalloc(ptr, bytes);
    };
    A((void**)&sl->work, (np / 2) * sizeof(float2));
    A((void**)&sl->work2, (np / 2) * sizeof(float2));
    A((void**)&sl->spec, (np32 / 2) * sizeof(float2));
    A((void**)&sl->planes, np32 / 8 + 256);
    A((void**)&sl->err, sizeof(int));
    A((void**)&sl->cnt, 2 * sizeof(unsigned long long));
    A((void**)&sl->resid, sizeof(unsigned int));
    A((void**)&sl->seed, words * 4);
    A((void**)&sl->ks, words * 4);
    A((void**)&sl->kr, words * 4);
    A((void**)&sl->out, words * 4);
    if (err == cudaSuccess) err = cudaMallocHost((void**)&sl->host, sizeof(Mirror));
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&sl->s, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&sl->join, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaMemset(sl->err, 0, sizeof(int));
    sl->bytes = slot_bytes(cap);
    p->used += sl->bytes;
    if (err != cudaSuccess) {
        free_slot(p, sl);
        return cuda_fail(e, err);
    }
    *out = sl;
    return PA_OK;
}

Pool* get_pool(pa_engine* e) {
    if (e->pool) return e->pool;
    Pool* p = new (std::nothrow) Pool();
    if (!p) return nullptr;
    if (cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&p->b0) != cudaSuccess || cudaEventCreate(&p->b1) != cudaSuccess) {
        delete p;
        return nullptr;
    }
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    p->budget = (uint64_t)(0.6 * (double)fr);
    e->pool = p;
    return p;
}

void drop_lane_graphs(LaneSet* ls) {
    if (!ls) return;
    for (auto& kv : ls->graphs) {
        cudaGraphExecDestroy(kv.second.exec);
        cudaFree(kv.second.jobs);
    }
    ls->graphs.clear();
}

void drop_graphs(Pool* p) {
    for (auto& kv : p->graphs) cudaGraphExecDestroy(kv.second);
    p->graphs.clear();
    for (auto& kv : p->graph_entries) cudaFree(kv.second);
    p->graph_entries.clear();
    drop_lane_graphs(p->lanes);
}

void free_gbuf(Pool* p, GroupBuf& gb) {
    cudaFree(gb.work);
    cudaFree(gb.work2);
    cudaFree(gb.spec);
    cudaFree(gb.planes);
    p->used -= std::min(p->used, gb.bytes);
    gb = GroupBuf{};
}

void free_lanes(Pool* p) {
    LaneSet* ls = p->lanes;
    if (!ls) return;
    cudaDeviceSynchronize();
    drop_lane_graphs(ls);
    cudaFree(ls->work);
    cudaFree(ls->work2);
    cudaFree(ls->spec);
    cudaFree(ls->planes);
    cudaFree(ls->maps);
    cudaFree(ls->ctl);
    cudaFree(ls->jobs);
    for (auto& kv : ls->spectra) {
        cudaFree(kv.second.spec);
        cudaFree(kv.second.cnt);
        p->used -= std::min(p->used, kv.second.bytes);
    }
    p->used -= std::min(p->used, ls->bytes);
    delete ls;
    p->lanes = nullptr;
}

int ensure_slot_maps(pa_engine* e, Slot* sl, const BlockGeom& g) {
    if (g.log_n1 == 0 || sl->maps_key == maps_key(g)) return PA_OK;
    int rc = pa::make_pass_maps(g, sl->work, sl->work2, &sl->maps);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    sl->maps_key = maps_key(g);
    return PA_OK;
}

pa::Scratch slot_scratch(Slot* sl) { return {sl->work, sl->work2, sl->planes, sl->err, &sl->maps}; }

int seed_in_slot(pa_engine* e, Slot* sl, const BlockGeom& g, const uint32_t* d_seed, float2* spec,
                 unsigned long long* cnt_seed, cudaStream_t s) {
    int rc = ensure_slot_maps(e, sl, g);
    if (rc) return rc;
    rc = pa::launch_seed_spectrum(g, d_seed, spec, slot_scratch(sl), cnt_seed, e->num_sms, s);
    return rc ? cuda_fail(e, (cudaError_t)rc) : PA_OK;
}

int key_in_slot(pa_engine* e, Slot* sl, const BlockGeom& g, const uint32_t* ks, const uint32_t* kr, uint32_t flags,
                const float2* spec, unsigned long long* cnt, unsigned int* resid, uint32_t* out, cudaStream_t s) {
    int rc = ensure_slot_maps(e, sl, g);
    if (rc) return rc;
    rc = pa::launch_key_block(g, ks, kr, flags, spec, slot_scratch(sl), cnt, resid, out, e->num_sms, s, nullptr);
    return rc ? cuda_fail(e, (cudaError_t)rc) : PA_OK;
}

// Exact recompute of one block in a slot (its spectrum buffer holds the seed transform).
int exact_in_slot(pa_engine* e, Slot* sl, const BlockGeom& g, const uint32_t* d_seed, const uint32_t* ks,
                  const uint32_t* kr, uint32_t flags, uint32_t* out, cudaStream_t s) {
    uint32_t* hat = reinterpret_cast<uint32_t*>(sl->spec);
    uint32_t* a = reinterpret_cast<uint32_t*>(sl->work);
    uint32_t* tmp = reinterpret_cast<uint32_t*>(sl->work2);
    int rc = pa::launch_exact_seed(g, d_seed, hat, tmp, &sl->ntt, s);
    if (!rc) rc = pa::launch_exact_block(g, ks, kr, flags, hat, a, tmp, out, &sl->ntt, s);
    return rc ? cuda_fail(e, (cudaError_t)rc) : PA_OK;
}

// Geometry of a job under the engine's split table, or under the split of its cached spectrum.
int job_geom(pa_engine* e, Pool* p, const pa_job& j, BlockGeom* g) {
    if (!j.key_start || !j.out) return PA_ERR_INVALID_ARG;
    if ((j.flags & PA_FLAG_XOR_KEY_REST) && !j.key_rest) return PA_ERR_INVALID_ARG;
    if (j.flags & PA_FLAG_EXACT) return PA_ERR_INVALID_ARG;
    int rc = make_geom(j.n, j.v, j.flags, e->split, g);
    if (rc) return rc;
    if (g->exact_only || g->log_np > kFp32MaxLogNp) return PA_ERR_TOO_LARGE;
    if (j.seed_id >= 0) {
        if ((size_t)j.seed_id >= p->seeds.size() || !p->seeds[j.seed_id].live) return PA_ERR_NO_SEED;
        const BlockGeom& sg = p->seeds[j.seed_id].g;
        if (g->log_n1 && sg.log_n == g->log_n) {
            g->log_n2 = sg.log_n2;
            g->log_n1 = sg.log_n - sg.log_n2;
        }
        if (!same_seed_geom(sg, *g)) return PA_ERR_INVALID_ARG;
    } else if (!j.seed_words) {
        return PA_ERR_NO_SEED;
    }
    return PA_OK;
}

bool any_busy(Pool* p) {
    for (Slot* sl : p->slots)
        if (sl->busy) return true;
    return false;
}

// Frees the group working sets, then idle slots (least recently used first), until `need` more bytes
// fit the budget.
bool make_room(Pool* p, size_t need) {
    while (p->used + need > p->budget) {
        if (!p->batch_pending) {  // group working sets first: only a pending batch uses them
            bool freed = false;
            for (GroupBuf& gb : p->gbufs)
                if (gb.bytes) {
                    free_gbuf(p, gb);
                    freed = true;
                }
            if (freed) {
                drop_graphs(p);
                continue;
            }
        }
        Slot* victim = nullptr;
        for (Slot* sl : p->slots)
            if (!sl->busy && (!victim || sl->last_use < victim->last_use)) victim = sl;
        if (!victim) return false;
        p->slots.erase(std::find(p->slots.begin(), p->slots.end(), victim));
        free_slot(p, victim);
        drop_graphs(p);
    }
    return true;
}

uint64_t fnv(uint64_t h, const void* data, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

double job_cost(const BlockGeom& g, bool dynamic) {
    const double np = double(1ull << g.log_np);
    return np * g.log_np * (dynamic ? 1.6 : 1.0);
}

// order[k]: what slot k runs, a job index or -(group + 1); entries: the device copy of p->hentries.
int batch_enqueue(pa_engine* e, Pool* p, const std::vector<std::vector<int>>& order, cudaStream_t s,
                  const pa::GroupEntry* entries) {
    PA_CUDA(e, cudaEventRecord(p->fork, s));
    for (size_t k = 0; k < order.size(); ++k) {
        Slot* sl = p->slots[k];
        PA_CUDA(e, cudaStreamWaitEvent(sl->s, p->fork, 0));
        for (int j : order[k]) {
            if (j < 0) {  // a group: one launch per pass for all its blocks
                const GroupChunk& ch = p->chunks[(size_t)(-j - 1)];
                const GroupBuf& gb = p->gbufs[(size_t)(-j - 1)];
                const pa::Group gp{entries + ch.entry_off, ch.count, size_t(1) << ch.g.log_n,
                                   group_planes_stride(ch.g)};
                const pa::Scratch sc{gb.work, gb.work2, gb.planes, sl->err, &ch.maps};
                int rc = pa::launch_group_prep(gp, sl->s);
                if (!rc && ch.dynamic) rc = pa::launch_group_seed(ch.g, gp, gb.spec, sc, e->num_sms, sl->s);
                if (!rc) rc = pa::launch_group_key(ch.g, gp, ch.flags, sc, e->num_sms, sl->s);
                if (rc) return cuda_fail(e, (cudaError_t)rc);
                continue;
            }
            const pa_job& jb = p->jobs[j];
            const BlockGeom& g = p->geoms[j];
            unsigned long long* cnt = p->job_cnt + 2 * (size_t)j;
            unsigned int* resid = p->job_resid + j;
            const float2* spec;
            int rc;
            if (jb.seed_id >= 0) {
                const SeedEntry& se = p->seeds[jb.seed_id];
                PA_CUDA(e, cudaMemcpyAsync(cnt + 1, se.cnt, sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                                           sl->s));
                spec = se.spec;
            } else {
                rc = seed_in_slot(e, sl, g, jb.seed_words, sl->spec, cnt + 1, sl->s);
                if (rc) return rc;
                spec = sl->spec;
            }
            rc = key_in_slot(e, sl, g, jb.key_start, jb.key_rest, jb.flags, spec, cnt, resid,
                             reinterpret_cast<uint32_t*>(jb.out), sl->s);
            if (rc) return rc;
        }
        PA_CUDA(e, cudaEventRecord(sl->join, sl->s));
        PA_CUDA(e, cudaStreamWaitEvent(s, sl->join, 0));
    }
    return PA_OK;
}

// Groups of a batch: jobs of one geometry (same n, v, flags and split; all static or all with their own
// seed; single-CTA blocks too), p->min_group or more, cut into groups of at most 2^p->group_log_bits bits of cyclic
// length (larger blocks run alone).  Fills p->chunks and p->hentries, sizes the group buffers (reallocating
// one drops the captured graphs, which point into it) and marks the grouped jobs.  Groups nothing when
// the buffers would not fit the HBM budget.
int plan_groups(pa_engine* e, Pool* p, const pa_job* jobs, uint32_t count, const std::vector<BlockGeom>& geoms,
                std::vector<char>& grouped) {
    p->chunks.clear();
    p->hentries.clear();
    std::map<std::array<uint64_t, 4>, std::vector<int>> by;
    for (uint32_t i = 0; i < count; ++i) {
        const BlockGeom& g = geoms[i];
        if (g.log_np >= p->group_log_bits) continue;
        by[{((uint64_t)g.n << 32) | g.v, jobs[i].flags, (uint64_t)g.log_n2, jobs[i].seed_id < 0 ? 1ull : 0ull}]
            .push_back((int)i);
    }
    for (auto& kv : by) {
        const std::vector<int>& list = kv.second;
        if (list.size() < p->min_group) continue;
        const BlockGeom& g = geoms[list[0]];
        const size_t per = size_t(1) << (p->group_log_bits - g.log_np);
        for (size_t o = 0; o < list.size(); o += per) {
            const size_t cnt = std::min(per, list.size() - o);
            if (cnt < 2) break;  // a last single block runs alone
            GroupChunk ch;
            ch.g = g;
            ch.flags = jobs[list[0]].flags;
            ch.dynamic = jobs[list[0]].seed_id < 0;
            ch.count = (uint32_t)cnt;
            ch.entry_off = p->hentries.size();
            for (size_t b = 0; b < cnt; ++b) {
                const int j = list[o + b];
                const pa_job& jb = jobs[j];
                pa::GroupEntry en{};
                en.key_start = jb.key_start;
                en.key_rest = jb.key_rest;
                en.out = reinterpret_cast<uint32_t*>(jb.out);
                en.cnt = p->job_cnt + 2 * (size_t)j;
                en.resid = p->job_resid + j;
                if (ch.dynamic) {
                    en.seed = jb.seed_words;  // spec: the group buffer's, below
                } else {
                    const SeedEntry& se = p->seeds[jb.seed_id];
                    en.spec = se.spec;
                    en.seed_cnt = se.cnt;
                }
                p->hentries.push_back(en);
                ch.jobs.push_back(j);
                ch.cost += job_cost(geoms[j], ch.dynamic);
            }
            p->chunks.push_back(ch);
        }
    }
    // working sets: group c uses buffer c
    size_t grow = 0;
    for (size_t c = 0; c < p->chunks.size(); ++c) {
        const GroupChunk& ch = p->chunks[c];
        const size_t w = (size_t)ch.count << ch.g.log_n, pl = (size_t)ch.count * group_planes_stride(ch.g);
        if (c >= p->gbufs.size() || p->gbufs[c].work_cap < w || p->gbufs[c].planes_cap < pl)
            grow += 3 * w * sizeof(float2) + pl * 4;
    }
    if (p->used + grow > p->budget) {  // no room: every block runs alone
        p->chunks.clear();
        p->hentries.clear();
        return PA_OK;
    }
    if (p->gbufs.size() < p->chunks.size()) p->gbufs.resize(p->chunks.size());
    for (size_t c = 0; c < p->chunks.size(); ++c) {
        GroupChunk& ch = p->chunks[c];
        GroupBuf& gb = p->gbufs[c];
        const size_t w = (size_t)ch.count << ch.g.log_n, pl = (size_t)ch.count * group_planes_stride(ch.g);
        if (gb.work_cap < w || gb.planes_cap < pl) {
            drop_graphs(p);
            const size_t wc = std::max(w, gb.work_cap), pc = std::max(pl, gb.planes_cap);
            free_gbuf(p, gb);
            cudaError_t err = cudaMalloc(&gb.work, wc * sizeof(float2));
            if (err == cudaSuccess) err = cudaMalloc(&gb.work2, wc * sizeof(float2));
            if (err == cudaSuccess) err = cudaMalloc(&gb.spec, wc * sizeof(float2));
            if (err == cudaSuccess) err = cudaMalloc(&gb.planes, pc * 4);
            if (err != cudaSuccess) {
                free_gbuf(p, gb);
                return cuda_fail(e, err);
            }
            gb.work_cap = wc;
            gb.planes_cap = pc;
            gb.bytes = 3 * wc * sizeof(float2) + pc * 4;
            p->used += gb.bytes;
        }
        if (ch.dynamic)
            for (uint32_t b = 0; b < ch.count; ++b)
                p->hentries[ch.entry_off + b].spec = gb.spec + ((size_t)b << ch.g.log_n);
        int rc = pa::make_group_maps(ch.g, gb.work, gb.work2, ch.count, &ch.maps);
        if (rc) return cuda_fail(e, (cudaError_t)rc);
        for (int j : ch.jobs) grouped[(size_t)j] = 1;
    }
    return PA_OK;
}

// Per-job popcount and residual words for `count` jobs.
int ensure_job_arrays(pa_engine* e, Pool* p, uint32_t count) {
    if (p->job_cap >= count) return PA_OK;
    cudaFree(p->job_cnt);
    cudaFree(p->job_resid);
    p->job_cnt = nullptr;
    p->job_resid = nullptr;
    p->job_cap = 0;
    drop_graphs(p);
    PA_CUDA(e, cudaMalloc(&p->job_cnt, (size_t)count * 2 * sizeof(unsigned long long)));
    PA_CUDA(e, cudaMalloc(&p->job_resid, (size_t)count * sizeof(unsigned int)));
    p->job_cap = count;
    return PA_OK;
}

// ---------------------------------------------------------------------------------------- lanes
// Block geometry on the lanes: rows of 2^14, the cyclic length at least 2^20 (pa_lanes.cuh).
int lane_geom(uint32_t n, uint32_t v, uint32_t flags, BlockGeom* g) {
    if (n < 1024u || (n & 31u) || (v & 31u) || v == 0 || v >= n) return PA_ERR_INVALID_ARG;
    g->n = n;
    g->v = v;
    g->h = n - v;
    g->out_bits = (flags & PA_FLAG_COMPRESS) ? v : n / 2u;
    const uint64_t need = is_pow2(n) ? n : std::max<uint64_t>(n, (uint64_t)g->out_bits + g->h);
    g->log_np = std::max(ceil_log2(need), pa::kLaneMinLogNp);
    if (g->log_np > pa::kLaneMaxLogNp) return PA_ERR_TOO_LARGE;
    const uint64_t np = 1ull << g->log_np;
    g->seed_direct = is_pow2(n) ? n : (uint32_t)std::min<uint64_t>(np - g->h, n);  // pow2: periodic placement
    g->log_n = g->log_np - 1;
    g->log_n2 = pa::kLaneLogRow;
    g->log_n1 = g->log_n - pa::kLaneLogRow;
    g->exact_only = 0;
    return PA_OK;
}

size_t lane_bytes(int cap) {
    const size_t np = size_t(1) << cap;
    return 3 * (np / 2) * sizeof(float2) + np / 8 + 256;
}

// Lanes of p->lane_ctas CTAs for cyclic lengths up to 2^cap: as many as fit the resident CTAs of the
// lane kernel and the HBM budget.
int ensure_lanes(pa_engine* e, Pool* p, int cap) {
    cap = std::max(cap, p->lane_cap);
    LaneSet* ls = p->lanes;
    if (ls && ls->cap >= cap && ls->T == p->lane_ctas) return PA_OK;
    free_lanes(p);
    int ctas = 0;
    int rc = pa::lane_max_ctas(&ctas);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    const int T = p->lane_ctas;
    int lanes = ctas / T;
    const size_t per = lane_bytes(cap);
    while (lanes > 0 && p->used + (size_t)lanes * per > p->budget) --lanes;
    if (lanes == 0) return PA_ERR_TOO_LARGE;
    ls = new (std::nothrow) LaneSet();
    if (!ls) return PA_ERR_INVALID_ARG;
    ls->T = T;
    ls->lanes = lanes;
    ls->cap = cap;
    ls->smem = pa::lane_smem_bytes();
    const size_t np = size_t(1) << cap;
    ls->work_stride = np / 2;
    ls->planes_stride = np / 32 + 64;
    cudaError_t err = cudaSuccess;
    auto A = [&](void** ptr, size_t bytes) {
        if (err == cudaSuccess) err = cudaMalloc(ptr, bytes);
    };
    A((void**)&ls->work, (size_t)lanes * ls->work_stride * sizeof(float2));
    A((void**)&ls->work2, (size_t)lanes * ls->work_stride * sizeof(float2));
    A((void**)&ls->spec, (size_t)lanes * ls->work_stride * sizeof(float2));
    A((void**)&ls->planes, (size_t)lanes * ls->planes_stride * sizeof(uint32_t));
    A((void**)&ls->maps, (size_t)lanes * pa::kLaneMaps * 2 * sizeof(CUtensorMap));
    A((void**)&ls->ctl, (1 + 3 * (size_t)lanes) * sizeof(unsigned int));
    ls->bytes = (size_t)lanes * per;
    p->used += ls->bytes;
    p->lanes = ls;
    if (err != cudaSuccess) {
        free_lanes(p);
        return cuda_fail(e, err);
    }
    std::vector<CUtensorMap> maps((size_t)lanes * pa::kLaneMaps * 2);
    for (int l = 0; l < lanes; ++l) {
        rc = pa::make_lane_maps(ls->work + (size_t)l * ls->work_stride, ls->work2 + (size_t)l * ls->work_stride,
                                maps.data() + (size_t)l * pa::kLaneMaps * 2);
        if (rc) {
            free_lanes(p);
            return cuda_fail(e, (cudaError_t)rc);
        }
    }
    err = cudaMemcpy(ls->maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
        free_lanes(p);
        return cuda_fail(e, err);
    }
    for (int i = 0; i < pa::kLaneMaps; ++i) {
        ls->early_b[i] = pa::lane_early_boxes(pa::kLaneMinLogN1 + i, 'b', ls->smem);
        ls->early_c[i] = pa::lane_early_boxes(pa::kLaneMinLogN1 + i, 'c', ls->smem);
    }
    return PA_OK;
}

// Key of a static seed's lane spectrum: the seed and its placement (a power-of-two n is placed
// periodically, so every v shares its spectrum).
std::array<uint64_t, 4> lane_spec_key(int32_t seed_id, const BlockGeom& g) {
    const bool identity = is_pow2(g.n);
    return {(uint64_t)seed_id, (uint64_t)g.log_np, identity ? 0ull : g.seed_direct, identity ? 0ull : g.h};
}

pa::LaneArgs lane_args(const LaneSet* ls, const pa::LaneJob* jobs, uint32_t njobs) {
    pa::LaneArgs a{};
    a.jobs = jobs;
    a.njobs = njobs;
    a.next = ls->ctl;
    a.bar = ls->ctl + 1;
    a.slot = reinterpret_cast<int*>(ls->ctl + 1 + ls->lanes);
    a.err = reinterpret_cast<int*>(ls->ctl + 1 + 2 * ls->lanes);
    a.work = ls->work;
    a.work2 = ls->work2;
    a.spec = ls->spec;
    a.planes = ls->planes;
    a.work_stride = ls->work_stride;
    a.planes_stride = ls->planes_stride;
    a.maps = ls->maps;
    a.T = ls->T;
    a.lanes = ls->lanes;
    for (int i = 0; i < pa::kLaneMaps; ++i) {
        a.early_b[i] = ls->early_b[i];
        a.early_c[i] = ls->early_c[i];
    }
    a.wait_limit = 1u << 24;  // polls of ~0.1-1 us: seconds, far beyond any stage of a 2^27 block
    return a;
}

// Queues one lane launch over `jobs` (uploaded to the lane set's job array).
int lanes_launch(pa_engine* e, LaneSet* ls, const std::vector<pa::LaneJob>& jobs, cudaStream_t s) {
    if (ls->job_cap < jobs.size()) {
        cudaFree(ls->jobs);
        ls->jobs = nullptr;
        ls->job_cap = 0;
        PA_CUDA(e, cudaMalloc(&ls->jobs, jobs.size() * sizeof(pa::LaneJob)));
        ls->job_cap = (uint32_t)jobs.size();
    }
    PA_CUDA(e, cudaMemcpyAsync(ls->jobs, jobs.data(), jobs.size() * sizeof(pa::LaneJob), cudaMemcpyHostToDevice, s));
    PA_CUDA(e, cudaMemsetAsync(ls->ctl, 0, (1 + 3 * (size_t)ls->lanes) * sizeof(unsigned int), s));
    const pa::LaneArgs a = lane_args(ls, ls->jobs, (uint32_t)jobs.size());
    int rc = pa::launch_lanes(a, ls->lanes * ls->T, ls->smem, s);
    return rc ? cuda_fail(e, (cudaError_t)rc) : PA_OK;
}

// The batch on the lanes: lane spectra of new static seeds first (one launch), then the blocks, longest
// first (one launch, or its captured graph with PA_BATCH_GRAPH).
int lanes_batch(pa_engine* e, Pool* p, const pa_job* jobs, uint32_t count, uint32_t batch_flags, cudaStream_t s) {
    std::vector<BlockGeom> lg(count);
    int cap = pa::kLaneMinLogNp;
    for (uint32_t i = 0; i < count; ++i) {
        int rc = lane_geom(jobs[i].n, jobs[i].v, jobs[i].flags, &lg[i]);
        if (rc) return rc;
        cap = std::max(cap, lg[i].log_np);
    }
    int rc = ensure_lanes(e, p, cap);
    if (rc) return rc;
    LaneSet* ls = p->lanes;
    std::vector<pa::LaneJob> builds;
    for (uint32_t i = 0; i < count; ++i) {
        if (jobs[i].seed_id < 0) continue;
        const auto key = lane_spec_key(jobs[i].seed_id, lg[i]);
        if (ls->spectra.count(key)) continue;
        LaneSpec sp;
        sp.bytes = (size_t(1) << lg[i].log_n) * sizeof(float2) + 32;
        if (p->used + sp.bytes > p->budget) return PA_ERR_TOO_LARGE;
        cudaError_t err = cudaMalloc(&sp.spec, (size_t(1) << lg[i].log_n) * sizeof(float2));
        if (err == cudaSuccess) err = cudaMalloc(&sp.cnt, 4 * sizeof(unsigned long long));
        if (err != cudaSuccess) {
            cudaFree(sp.spec);
            return cuda_fail(e, err);
        }
        p->used += sp.bytes;
        ls->spectra[key] = sp;
        pa::LaneJob b{};
        b.seed = p->seeds[jobs[i].seed_id].seed;
        b.spec_out = sp.spec;
        b.cnt = sp.cnt;
        b.resid = reinterpret_cast<unsigned int*>(sp.cnt + 2);
        b.g = lg[i];
        builds.push_back(b);
    }
    if (!builds.empty()) {
        drop_lane_graphs(ls);
        rc = lanes_launch(e, ls, builds, s);
        if (rc) return rc;
    }
    std::vector<int> idx(count);
    std::iota(idx.begin(), idx.end(), 0);
    std::vector<double> cost(count);
    for (uint32_t i = 0; i < count; ++i) cost[i] = job_cost(lg[i], jobs[i].seed_id < 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<pa::LaneJob> lj(count);
    for (uint32_t k = 0; k < count; ++k) {
        const int i = idx[k];
        const pa_job& jb = jobs[i];
        pa::LaneJob& j = lj[k];
        j.key_start = jb.key_start;
        j.key_rest = (jb.flags & PA_FLAG_XOR_KEY_REST) ? jb.key_rest : nullptr;
        if (jb.seed_id >= 0) {
            const LaneSpec& sp = ls->spectra[lane_spec_key(jb.seed_id, lg[i])];
            j.spec = sp.spec;
            j.seed_cnt = sp.cnt + 1;
        } else {
            j.seed = jb.seed_words;
        }
        j.out = reinterpret_cast<uint32_t*>(jb.out);
        j.cnt = p->job_cnt + 2 * (size_t)i;
        j.resid = p->job_resid + i;
        j.g = lg[i];
        j.flags = jb.flags;
    }
    PA_CUDA(e, cudaEventRecord(p->b0, s));
    if (batch_flags & PA_BATCH_GRAPH) {
        uint64_t key = fnv(1469598103934665603ull, lj.data(), lj.size() * sizeof(pa::LaneJob));
        auto it = ls->graphs.find(key);
        if (it == ls->graphs.end()) {
            LaneGraph lgph;
            PA_CUDA(e, cudaMalloc(&lgph.jobs, lj.size() * sizeof(pa::LaneJob)));
            PA_CUDA(e, cudaMemcpy(lgph.jobs, lj.data(), lj.size() * sizeof(pa::LaneJob), cudaMemcpyHostToDevice));
            PA_CUDA(e, cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            cudaError_t cerr = cudaMemsetAsync(ls->ctl, 0, (1 + 3 * (size_t)ls->lanes) * sizeof(unsigned int), s);
            int lrc = cerr == cudaSuccess
                          ? pa::launch_lanes(lane_args(ls, lgph.jobs, count), ls->lanes * ls->T, ls->smem, s)
                          : (int)cerr;
            cudaGraph_t graph = nullptr;
            cerr = cudaStreamEndCapture(s, &graph);
            if (lrc || cerr != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                cudaFree(lgph.jobs);
                return cuda_fail(e, lrc ? (cudaError_t)lrc : cerr);
            }
            cerr = cudaGraphInstantiate(&lgph.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (cerr != cudaSuccess) {
                cudaFree(lgph.jobs);
                return cuda_fail(e, cerr);
            }
            if (ls->graphs.size() >= 16) drop_lane_graphs(ls);
            it = ls->graphs.emplace(key, lgph).first;
        }
        PA_CUDA(e, cudaGraphLaunch(it->second.exec, s));
    } else {
        rc = lanes_launch(e, ls, lj, s);
        if (rc) return rc;
    }
    PA_CUDA(e, cudaEventRecord(p->b1, s));
    return PA_OK;
}

// ---------------------------------------------------------------------------------- serving loop
void free_serve(Pool* p) {
    ServeLoop* sv = p->serve;
    if (!sv) return;
    if (sv->ctl) sv->ctl->stop = 1;
    if (sv->launched) cudaEventSynchronize(sv->ended);  // the loop ends once it sees stop (bounded)
    if (sv->s) cudaStreamSynchronize(sv->s);
    cudaFreeHost(sv->ring);
    cudaFreeHost(sv->ctl);
    cudaFree(sv->claimed);
    cudaFree(sv->lane_job);
    cudaFree(sv->lane_stats);
    cudaFree(sv->stage);
    if (sv->ended) cudaEventDestroy(sv->ended);
    if (sv->s) cudaStreamDestroy(sv->s);
    delete sv;
    p->serve = nullptr;
}

// Whether the last launch of the loop left a lane error word set (a bounded wait expired).
int serve_lane_error(pa_engine* e, Pool* p, bool* any) {
    std::vector<int> lerr(p->lanes->lanes);
    PA_CUDA(e, cudaMemcpy(lerr.data(), p->lanes->ctl + 1 + 2 * p->lanes->lanes, lerr.size() * sizeof(int),
                          cudaMemcpyDeviceToHost));
    *any = false;
    for (int x : lerr) *any = *any || x != 0;
    return PA_OK;
}

// (Re)launches the serving loop on the lanes; `claimed` keeps counting across launches.  A loop whose last
// launch ended with a lane error is not launched again: it stays failed until pa_serve_stop.
int serve_launch(pa_engine* e, Pool* p) {
    ServeLoop* sv = p->serve;
    LaneSet* ls = p->lanes;
    if (sv->launched) {
        bool bad = false;
        int rc = serve_lane_error(e, p, &bad);
        if (rc) return rc;
        if (bad) sv->failed = true;
    }
    if (sv->failed) {
        e->last_cuda = (int)cudaErrorLaunchTimeout;
        return PA_ERR_CUDA;
    }
    PA_CUDA(e, cudaMemsetAsync(ls->ctl, 0, (1 + 3 * (size_t)ls->lanes) * sizeof(unsigned int), sv->s));
    pa::LaneArgs a = lane_args(ls, nullptr, 0);
    a.serve = 1;
    a.ring = sv->d_ring;
    a.ring_size = sv->size;
    a.host = sv->d_ctl;
    a.claimed = sv->claimed;
    a.lane_job = sv->lane_job;
    a.lane_stats = sv->lane_stats;
    a.stage = sv->stage;
    a.stage_stride = sv->stage_stride;
    a.idle_ns = sv->idle_ns;
    int rc = pa::launch_lanes(a, ls->lanes * ls->T, ls->smem, sv->s);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    PA_CUDA(e, cudaEventRecord(sv->ended, sv->s));
    sv->launched = true;
    return PA_OK;
}

bool serve_running(ServeLoop* sv) { return sv->launched && cudaEventQuery(sv->ended) == cudaErrorNotReady; }

// The address the device uses for a served request's buffer: device or managed memory as it is, pinned
// host memory through its device mapping; anything else (pageable memory) is refused, since the lanes
// read and write these buffers directly.
bool device_view(const void* p, const void** out) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        *out = p;
        return true;
    }
    if (at.type == cudaMemoryTypeHost && at.devicePointer) {
        *out = at.devicePointer;
        return true;
    }
    return false;
}

// A slot for an exact recompute of a block of cyclic length 2^cap (one is made if none is idle).
int exact_slot(pa_engine* e, Pool* p, int cap, Slot** out) {
    for (Slot* c : p->slots)
        if (!c->busy && c->cap >= cap) {
            *out = c;
            return PA_OK;
        }
    if (!make_room(p, slot_bytes(cap))) return PA_ERR_TOO_LARGE;
    Slot* sl = nullptr;
    int rc = new_slot(e, p, cap, &sl);
    if (rc) return rc;
    sl->last_use = ++p->clock;
    p->slots.push_back(sl);
    *out = sl;
    return PA_OK;
}

}  // namespace

void pool_destroy(pa_engine* e) {
    Pool* p = e->pool;
    if (!p) return;
    free_serve(p);
    drop_graphs(p);
    free_lanes(p);
    for (Slot* sl : p->slots) free_slot(p, sl);
    for (auto& se : p->seeds) {
        cudaFree(se.spec);
        cudaFree(se.seed);
        cudaFree(se.cnt);
    }
    cudaFree(p->job_cnt);
    cudaFree(p->job_resid);
    for (GroupBuf& gb : p->gbufs) free_gbuf(p, gb);
    cudaFree(p->gentries);
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->b0) cudaEventDestroy(p->b0);
    if (p->b1) cudaEventDestroy(p->b1);
    delete p;
    e->pool = nullptr;
}

}  // namespace pa_host

using namespace pa_host;

extern "C" {

int pa_set_pool(pa_engine* e, uint64_t hbm_budget_bytes, int32_t max_slots, int32_t batch_slots) {
    if (!e || max_slots < 0 || batch_slots < 0 || max_slots > 256 || batch_slots > 256) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (hbm_budget_bytes) p->budget = hbm_budget_bytes;
    p->max_slots = max_slots ? max_slots : 16;
    p->batch_slots = batch_slots ? batch_slots : 8;
    drop_graphs(p);
    return PA_OK;
}

int pa_set_groups(pa_engine* e, int32_t min_blocks, int32_t log_bits) {
    if (!e || min_blocks < 0 || log_bits < 0 || (min_blocks && min_blocks < 2) || (log_bits && (log_bits < 17 || log_bits > 30)))
        return PA_ERR_INVALID_ARG;
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (p->batch_pending) return PA_ERR_BUSY;
    p->min_group = min_blocks ? (uint32_t)min_blocks : kMinGroup;
    p->group_log_bits = log_bits ? log_bits : kGroupLogBits;
    drop_graphs(p);
    return PA_OK;
}

int pa_set_lanes(pa_engine* e, int32_t ctas_per_lane, uint32_t max_np) {
    if (!e || ctas_per_lane < 0 || ctas_per_lane > 1024) return PA_ERR_INVALID_ARG;
    if (max_np && (max_np & (max_np - 1u))) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (p->batch_pending || p->serve) return PA_ERR_BUSY;
    const int cap = max_np ? ceil_log2(max_np) : 0;
    if (cap > pa::kLaneMaxLogNp) return PA_ERR_TOO_LARGE;
    const int T = ctas_per_lane ? ctas_per_lane : 4;
    if (p->lanes && (p->lanes->T != T || p->lanes->cap < cap)) free_lanes(p);
    p->lane_ctas = T;
    p->lane_cap = cap;
    if (cap) {
        int rc = ensure_lanes(e, p, cap);
        if (rc) return rc;
    }
    return p->lanes ? p->lanes->lanes : 0;
}

int pa_pool_reserve(pa_engine* e, uint32_t max_np, int32_t count) {
    if (!e || count < 0 || max_np < 1024u || (max_np & (max_np - 1u))) return PA_ERR_INVALID_ARG;
    const int cap = ceil_log2(max_np);
    if (cap > kFp32MaxLogNp) return PA_ERR_TOO_LARGE;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    int have = 0;
    for (Slot* c : p->slots) have += c->cap >= cap ? 1 : 0;
    while (have < count && (int)p->slots.size() < p->max_slots) {
        if (p->used + slot_bytes(cap) > p->budget) break;
        Slot* sl = nullptr;
        int rc = new_slot(e, p, cap, &sl);
        if (rc) return rc;
        sl->last_use = ++p->clock;
        p->slots.push_back(sl);
        ++have;
    }
    drop_graphs(p);
    return have;
}

int pa_seed_cache_add(pa_engine* e, const uint32_t* seed_words, uint32_t n, uint32_t v, uint32_t flags,
                      int32_t* seed_id) {
    if (!e || !seed_words || !seed_id) return PA_ERR_INVALID_ARG;
    BlockGeom g;
    int rc = make_geom(n, v, flags & ~PA_FLAG_EXACT, e->split, &g);
    if (rc) return rc;
    if (g.exact_only || g.log_np > kFp32MaxLogNp) return PA_ERR_TOO_LARGE;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (any_busy(p) || p->batch_pending) return PA_ERR_BUSY;
    SeedEntry se;
    se.g = g;
    const size_t words = n / 32u;
    se.bytes = (size_t(1) << g.log_n) * sizeof(float2) + words * 4 + 8;
    if (!make_room(p, se.bytes)) return PA_ERR_TOO_LARGE;
    cudaError_t err = cudaMalloc(&se.spec, (size_t(1) << g.log_n) * sizeof(float2));
    if (err == cudaSuccess) err = cudaMalloc(&se.seed, words * 4);
    if (err == cudaSuccess) err = cudaMalloc(&se.cnt, sizeof(unsigned long long));
    if (err == cudaSuccess) err = cudaMemcpy(se.seed, seed_words, words * 4, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
        cudaFree(se.spec);
        cudaFree(se.seed);
        cudaFree(se.cnt);
        return cuda_fail(e, err);
    }
    // build in any idle slot large enough (or a temporary one)
    Slot* sl = nullptr;
    for (Slot* c : p->slots)
        if (!c->busy && c->cap >= g.log_np && (!sl || c->cap < sl->cap)) sl = c;
    Slot* tmp = nullptr;
    if (!sl) {
        if (!make_room(p, slot_bytes(g.log_np))) rc = PA_ERR_TOO_LARGE;
        else rc = new_slot(e, p, g.log_np, &tmp);
        sl = tmp;
    }
    if (!rc) rc = seed_in_slot(e, sl, g, se.seed, se.spec, se.cnt, sl->s);
    if (!rc && cudaStreamSynchronize(sl->s) != cudaSuccess) rc = PA_ERR_CUDA;
    int derr = 0;
    if (!rc && cudaMemcpy(&derr, sl->err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && derr) {
        cudaMemset(sl->err, 0, sizeof(int));
        e->last_cuda = (int)cudaErrorLaunchTimeout;
        rc = PA_ERR_CUDA;
    }
    if (tmp) {
        if ((int)p->slots.size() < p->max_slots) {  // keep it: blocks of this size will want it
            tmp->last_use = ++p->clock;
            p->slots.push_back(tmp);
        } else {
            free_slot(p, tmp);
        }
    }
    if (rc) {
        cudaFree(se.spec);
        cudaFree(se.seed);
        cudaFree(se.cnt);
        return rc;
    }
    se.live = true;
    p->used += se.bytes;
    p->seeds.push_back(se);
    *seed_id = (int32_t)(p->seeds.size() - 1);
    return PA_OK;
}

int pa_seed_cache_clear(pa_engine* e) {
    if (!e) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = e->pool;
    if (!p) return PA_OK;
    if (any_busy(p) || p->batch_pending) return PA_ERR_BUSY;
    drop_graphs(p);
    for (auto& se : p->seeds) {
        cudaFree(se.spec);
        cudaFree(se.seed);
        cudaFree(se.cnt);
        p->used -= std::min(p->used, se.bytes);
    }
    p->seeds.clear();
    return PA_OK;
}

int pa_batch_run(pa_engine* e, const pa_job* jobs, uint32_t count, uint32_t batch_flags, void* stream) {
    if (!e || (!jobs && count)) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (any_busy(p) || p->batch_pending) return PA_ERR_BUSY;
    if (p->serve && (batch_flags & PA_BATCH_PERSISTENT)) return PA_ERR_BUSY;  // the lanes are serving
    std::vector<BlockGeom> geoms(count);
    int need_cap = 0;
    for (uint32_t i = 0; i < count; ++i) {
        int rc = job_geom(e, p, jobs[i], &geoms[i]);
        if (rc) return rc;
        if (reinterpret_cast<uintptr_t>(jobs[i].out) & 3u) return PA_ERR_INVALID_ARG;
        need_cap = std::max(need_cap, geoms[i].log_np);
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    p->batch_stream = s;
    p->jobs.assign(jobs, jobs + count);
    p->geoms = geoms;
    if (count == 0) {
        PA_CUDA(e, cudaEventRecord(p->b0, s));
        PA_CUDA(e, cudaEventRecord(p->b1, s));
        p->batch_pending = true;
        return PA_OK;
    }
    if (batch_flags & PA_BATCH_PERSISTENT) {
        int rc = ensure_job_arrays(e, p, count);
        if (!rc) rc = lanes_batch(e, p, jobs, count, batch_flags, s);
        if (rc) return rc;
        p->batch_lanes = true;
        p->batch_pending = true;
        return PA_OK;
    }
    p->batch_lanes = false;
    int K = (batch_flags & PA_BATCH_SERIAL) ? 1 : std::min<int>(p->batch_slots, (int)count);
    K = std::min(K, p->max_slots);
    // slots 0..K-1 must hold the largest block of the batch
    for (int k = 0; k < K; ++k) {
        if (k < (int)p->slots.size() && p->slots[k]->cap >= need_cap) continue;
        if (k < (int)p->slots.size()) {
            Slot* old = p->slots[k];
            p->slots.erase(p->slots.begin() + k);
            free_slot(p, old);
            drop_graphs(p);
        }
        Slot* sl = nullptr;
        // free idle slots beyond K first, then give up on parallelism if HBM is short
        while (p->used + slot_bytes(need_cap) > p->budget && (int)p->slots.size() > k) {
            Slot* victim = p->slots.back();
            p->slots.pop_back();
            free_slot(p, victim);
            drop_graphs(p);
        }
        if (p->used + slot_bytes(need_cap) > p->budget) {
            if (k == 0) return PA_ERR_TOO_LARGE;
            K = k;
            break;
        }
        int rc = new_slot(e, p, need_cap, &sl);
        if (rc) return rc;
        p->slots.insert(p->slots.begin() + k, sl);
    }
    {
        int rc = ensure_job_arrays(e, p, count);
        if (rc) return rc;
    }
    // groups of equal blocks, then every unit (a job alone or a group) longest first onto the
    // least-loaded slot
    std::vector<char> grouped(count, 0);
    if (!(batch_flags & (PA_BATCH_SERIAL | PA_BATCH_NO_GROUP))) {
        int rc = plan_groups(e, p, jobs, count, geoms, grouped);
        if (rc) return rc;
    } else {
        p->chunks.clear();
        p->hentries.clear();
    }
    std::vector<int> units;
    std::vector<double> cost;
    for (uint32_t i = 0; i < count; ++i)
        if (!grouped[i]) {
            units.push_back((int)i);
            cost.push_back(job_cost(geoms[i], jobs[i].seed_id < 0));
        }
    for (size_t c = 0; c < p->chunks.size(); ++c) {
        units.push_back(-(int)c - 1);
        cost.push_back(p->chunks[c].cost);
    }
    std::vector<int> idx(units.size());
    std::iota(idx.begin(), idx.end(), 0);
    if (!(batch_flags & PA_BATCH_SERIAL))
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<std::vector<int>> order(K);
    std::vector<double> load(K, 0.0);
    for (int u : idx) {
        int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        order[k].push_back(units[u]);
        load[k] += cost[u];
    }
    // the groups' entry table (a pending batch finished before this one was accepted, so the table of a
    // run without a graph is free to overwrite)
    const size_t ne = p->hentries.size();
    if (ne && !(batch_flags & PA_BATCH_GRAPH)) {
        if (p->gentries_cap < ne) {
            cudaFree(p->gentries);
            p->gentries = nullptr;
            p->gentries_cap = 0;
            PA_CUDA(e, cudaMalloc(&p->gentries, ne * sizeof(pa::GroupEntry)));
            p->gentries_cap = ne;
        }
        PA_CUDA(e, cudaMemcpy(p->gentries, p->hentries.data(), ne * sizeof(pa::GroupEntry), cudaMemcpyHostToDevice));
    }
    for (int k = 0; k < K; ++k) p->slots[k]->last_use = ++p->clock;
    PA_CUDA(e, cudaEventRecord(p->b0, s));
    if (batch_flags & PA_BATCH_GRAPH) {
        uint64_t key = fnv(1469598103934665603ull, jobs, sizeof(pa_job) * count);
        key = fnv(key, &K, sizeof(K));
        key = fnv(key, &batch_flags, sizeof(batch_flags));
        for (const auto& g : geoms) key = fnv(key, &g, sizeof(g));
        auto it = p->graphs.find(key);
        if (it == p->graphs.end()) {
            if (p->graphs.size() >= 16) drop_graphs(p);
            pa::GroupEntry* table = nullptr;  // the graph's own copy of the entries
            if (ne) {
                PA_CUDA(e, cudaMalloc(&table, ne * sizeof(pa::GroupEntry)));
                cudaError_t cerr = cudaMemcpy(table, p->hentries.data(), ne * sizeof(pa::GroupEntry),
                                              cudaMemcpyHostToDevice);
                if (cerr != cudaSuccess) {
                    cudaFree(table);
                    return cuda_fail(e, cerr);
                }
            }
            cudaError_t cerr = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
            if (cerr != cudaSuccess) {
                cudaFree(table);
                return cuda_fail(e, cerr);
            }
            int rc = batch_enqueue(e, p, order, s, table);
            cudaGraph_t graph = nullptr;
            cerr = cudaStreamEndCapture(s, &graph);
            if (rc || cerr != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                cudaFree(table);
                return rc ? rc : cuda_fail(e, cerr);
            }
            cudaGraphExec_t exec = nullptr;
            cerr = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (cerr != cudaSuccess) {
                cudaFree(table);
                return cuda_fail(e, cerr);
            }
            it = p->graphs.emplace(key, exec).first;
            if (table) p->graph_entries[key] = table;
        }
        PA_CUDA(e, cudaGraphLaunch(it->second, s));
    } else {
        int rc = batch_enqueue(e, p, order, s, p->gentries);
        if (rc) return rc;
    }
    PA_CUDA(e, cudaEventRecord(p->b1, s));
    p->batch_pending = true;
    return PA_OK;
}

int pa_batch_sync(pa_engine* e, pa_stats* stats, uint32_t count) {
    if (!e) return PA_ERR_INVALID_ARG;
    Pool* p = e->pool;
    if (!p || !p->batch_pending) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    p->batch_pending = false;
    PA_CUDA(e, cudaStreamSynchronize(p->batch_stream));
    const uint32_t nj = (uint32_t)p->jobs.size();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->b0, p->b1);
    for (Slot* sl : p->slots) {
        int derr = 0;
        PA_CUDA(e, cudaMemcpy(&derr, sl->err, sizeof(int), cudaMemcpyDeviceToHost));
        if (derr) {  // a bounded device wait expired: results of this batch are not valid
            cudaMemset(sl->err, 0, sizeof(int));
            e->last_cuda = (int)cudaErrorLaunchTimeout;
            return PA_ERR_CUDA;
        }
    }
    if (p->batch_lanes && p->lanes) {  // lane error words: an expired lane barrier or TMA wait
        std::vector<int> lerr(p->lanes->lanes);
        PA_CUDA(e, cudaMemcpy(lerr.data(), p->lanes->ctl + 1 + 2 * p->lanes->lanes, lerr.size() * sizeof(int),
                              cudaMemcpyDeviceToHost));
        for (int x : lerr)
            if (x) {
                e->last_cuda = (int)cudaErrorLaunchTimeout;
                return PA_ERR_CUDA;
            }
    }
    if (nj == 0) return PA_OK;
    std::vector<unsigned long long> cnt(2 * (size_t)nj);
    std::vector<unsigned int> rb(nj);
    PA_CUDA(e, cudaMemcpy(cnt.data(), p->job_cnt, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    PA_CUDA(e, cudaMemcpy(rb.data(), p->job_resid, rb.size() * sizeof(unsigned int), cudaMemcpyDeviceToHost));
    for (uint32_t j = 0; j < nj; ++j) {
        float r;
        std::memcpy(&r, &rb[j], sizeof(r));
        int exact = 0;
        if (!(r <= e->residual_limit)) {  // FP32 budget exceeded: recompute this block exactly
            const pa_job& jb = p->jobs[j];
            const uint32_t* seed = jb.seed_id >= 0 ? p->seeds[jb.seed_id].seed : jb.seed_words;
            Slot* sl = nullptr;
            int rc = exact_slot(e, p, p->geoms[j].log_np, &sl);
            if (!rc)
                rc = exact_in_slot(e, sl, p->geoms[j], seed, jb.key_start, jb.key_rest, jb.flags,
                                   reinterpret_cast<uint32_t*>(jb.out), sl->s);
            if (rc) return rc;
            PA_CUDA(e, cudaStreamSynchronize(sl->s));
            exact = 1;
        }
        if (stats && j < count) {
            stats[j].max_residual = r;
            stats[j].popcount_key = cnt[2 * j];
            stats[j].popcount_seed = cnt[2 * j + 1];
            stats[j].gpu_ms = ms;
            stats[j].seed_uses_left = -1;
            stats[j].exact = exact;
        }
    }
    return PA_OK;
}

int pa_submit(pa_engine* e, const pa_job* job, uint64_t* ticket) {
    if (!e || !job || !ticket) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (p->batch_pending) return PA_ERR_BUSY;
    BlockGeom g;
    int rc = job_geom(e, p, *job, &g);
    if (rc) return rc;
    // at most max_slots blocks in flight; the smallest idle slot that holds the block, else a new
    // one within the budget (idle slots are freed, least recently used first, to make room)
    int busy = 0;
    for (Slot* c : p->slots) busy += c->busy ? 1 : 0;
    if (busy >= p->max_slots) return PA_ERR_BUSY;
    Slot* sl = nullptr;
    for (Slot* c : p->slots)
        if (!c->busy && c->cap >= g.log_np && (!sl || c->cap < sl->cap)) sl = c;
    if (!sl) {
        if ((int)p->slots.size() >= p->max_slots) {
            Slot* victim = nullptr;
            for (Slot* c : p->slots)
                if (!c->busy && (!victim || c->last_use < victim->last_use)) victim = c;
            if (!victim) return PA_ERR_BUSY;
            p->slots.erase(std::find(p->slots.begin(), p->slots.end(), victim));
            free_slot(p, victim);
            drop_graphs(p);
        }
        if (!make_room(p, slot_bytes(g.log_np))) return any_busy(p) ? PA_ERR_BUSY : PA_ERR_TOO_LARGE;
        rc = new_slot(e, p, g.log_np, &sl);
        if (rc) return rc;
        p->slots.push_back(sl);
    }
    const uint32_t n = job->n, v = job->v;
    cudaStream_t s = sl->s;
    const float2* spec;
    if (job->seed_id >= 0) {
        const SeedEntry& se = p->seeds[job->seed_id];
        PA_CUDA(e, cudaMemcpyAsync(sl->cnt + 1, se.cnt, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s));
        spec = se.spec;
    } else {
        PA_CUDA(e, cudaMemcpyAsync(sl->seed, job->seed_words, (size_t)(n / 32u) * 4u, cudaMemcpyHostToDevice, s));
        rc = seed_in_slot(e, sl, g, sl->seed, sl->spec, sl->cnt + 1, s);
        if (rc) return rc;
        spec = sl->spec;
    }
    PA_CUDA(e, cudaMemcpyAsync(sl->ks, job->key_start, (size_t)(g.h / 32u + 1u) * 4u, cudaMemcpyHostToDevice, s));
    if (job->flags & PA_FLAG_XOR_KEY_REST)
        PA_CUDA(e, cudaMemcpyAsync(sl->kr, job->key_rest, (size_t)(v / 32u) * 4u, cudaMemcpyHostToDevice, s));
    rc = key_in_slot(e, sl, g, sl->ks, sl->kr, job->flags, spec, sl->cnt, sl->resid, sl->out, s);
    if (rc) return rc;
    PA_CUDA(e, cudaMemcpyAsync(job->out, sl->out, pa_output_bytes(n, v, job->flags), cudaMemcpyDeviceToHost, s));
    PA_CUDA(e, cudaMemcpyAsync(sl->host->cnt, sl->cnt, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PA_CUDA(e, cudaMemcpyAsync(&sl->host->resid, sl->resid, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    PA_CUDA(e, cudaMemcpyAsync(&sl->host->err, sl->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    PA_CUDA(e, cudaEventRecord(sl->done, s));
    sl->busy = true;
    sl->ticket = p->next_ticket++;
    sl->job = *job;
    sl->g = g;
    sl->seed_id = job->seed_id;
    sl->last_use = ++p->clock;
    *ticket = sl->ticket;
    return PA_OK;
}

int pa_poll(pa_engine* e, uint64_t ticket, pa_stats* stats) {
    if (!e || !e->pool) return PA_ERR_INVALID_ARG;
    Pool* p = e->pool;
    Slot* sl = nullptr;
    for (Slot* c : p->slots)
        if (c->busy && c->ticket == ticket) sl = c;
    if (!sl) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    cudaError_t q = cudaEventQuery(sl->done);
    if (q == cudaErrorNotReady) return PA_PENDING;
    if (q != cudaSuccess) {
        sl->busy = false;
        return cuda_fail(e, q);
    }
    const Mirror m = *sl->host;
    if (m.err) {
        cudaMemset(sl->err, 0, sizeof(int));
        sl->busy = false;
        e->last_cuda = (int)cudaErrorLaunchTimeout;
        return PA_ERR_CUDA;
    }
    float r;
    std::memcpy(&r, &m.resid, sizeof(r));
    int exact = 0;
    if (!(r <= e->residual_limit)) {  // FP32 budget exceeded: recompute exactly, then copy out again
        const pa_job& jb = sl->job;
        const uint32_t* seed = sl->seed_id >= 0 ? p->seeds[sl->seed_id].seed : sl->seed;
        int rc = exact_in_slot(e, sl, sl->g, seed, sl->ks, sl->kr, jb.flags, sl->out, sl->s);
        if (!rc && cudaMemcpyAsync(jb.out, sl->out, pa_output_bytes(jb.n, jb.v, jb.flags), cudaMemcpyDeviceToHost,
                                   sl->s) != cudaSuccess)
            rc = PA_ERR_CUDA;
        if (!rc && cudaStreamSynchronize(sl->s) != cudaSuccess) rc = PA_ERR_CUDA;
        if (rc) {
            sl->busy = false;
            return rc;
        }
        exact = 1;
    }
    if (stats) {
        stats->max_residual = r;
        stats->popcount_key = m.cnt[0];
        stats->popcount_seed = m.cnt[1];
        stats->gpu_ms = 0.f;
        stats->seed_uses_left = -1;
        stats->exact = exact;
    }
    sl->busy = false;
    sl->last_use = ++p->clock;
    return PA_OK;
}

int pa_serve_start(pa_engine* e, int32_t ctas_per_lane, uint32_t max_np, int32_t ring_slots) {
    if (!e || ctas_per_lane < 0 || ring_slots < 0 || ring_slots > (1 << 20)) return PA_ERR_INVALID_ARG;
    if (!max_np || (max_np & (max_np - 1u))) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (p->serve || p->batch_pending || any_busy(p)) return PA_ERR_BUSY;
    const int cap = std::max(ceil_log2(max_np), pa::kLaneMinLogNp);
    if (cap > pa::kLaneMaxLogNp) return PA_ERR_TOO_LARGE;
    const int T = ctas_per_lane ? ctas_per_lane : 38;
    if (p->lanes && (p->lanes->T != T || p->lanes->cap < cap)) free_lanes(p);
    p->lane_ctas = T;
    int rc = ensure_lanes(e, p, cap);
    if (rc) return rc;
    LaneSet* ls = p->lanes;
    // lane spectra of every cached static seed, for its own geometry (one launch, synchronous)
    std::vector<pa::LaneJob> builds;
    for (size_t i = 0; i < p->seeds.size(); ++i) {
        const SeedEntry& se = p->seeds[i];
        if (!se.live) continue;
        BlockGeom lg;
        if (lane_geom(se.g.n, se.g.v, se.g.out_bits == se.g.v ? PA_FLAG_COMPRESS : 0u, &lg) || lg.log_np > ls->cap)
            continue;
        const auto key = lane_spec_key((int32_t)i, lg);
        if (ls->spectra.count(key)) continue;
        LaneSpec sp;
        sp.bytes = (size_t(1) << lg.log_n) * sizeof(float2) + 32;
        if (p->used + sp.bytes > p->budget) return PA_ERR_TOO_LARGE;
        cudaError_t err = cudaMalloc(&sp.spec, (size_t(1) << lg.log_n) * sizeof(float2));
        if (err == cudaSuccess) err = cudaMalloc(&sp.cnt, 4 * sizeof(unsigned long long));
        if (err != cudaSuccess) {
            cudaFree(sp.spec);
            return cuda_fail(e, err);
        }
        p->used += sp.bytes;
        ls->spectra[key] = sp;
        pa::LaneJob b{};
        b.seed = se.seed;
        b.spec_out = sp.spec;
        b.cnt = sp.cnt;
        b.resid = reinterpret_cast<unsigned int*>(sp.cnt + 2);
        b.g = lg;
        builds.push_back(b);
    }
    if (!builds.empty()) {
        rc = lanes_launch(e, ls, builds, e->stream);
        if (rc) return rc;
        PA_CUDA(e, cudaStreamSynchronize(e->stream));
    }
    ServeLoop* sv = new (std::nothrow) ServeLoop();
    if (!sv) return PA_ERR_INVALID_ARG;
    p->serve = sv;
    sv->size = ring_slots ? (uint32_t)ring_slots : 64u;
    cudaError_t err = cudaHostAlloc((void**)&sv->ring, sv->size * sizeof(pa::ServeSlot), cudaHostAllocMapped);
    if (err == cudaSuccess) err = cudaHostAlloc((void**)&sv->ctl, sizeof(pa::ServeCtl), cudaHostAllocMapped);
    if (err == cudaSuccess) err = cudaHostGetDevicePointer((void**)&sv->d_ring, sv->ring, 0);
    if (err == cudaSuccess) err = cudaHostGetDevicePointer((void**)&sv->d_ctl, sv->ctl, 0);
    if (err == cudaSuccess) err = cudaMalloc(&sv->claimed, sizeof(unsigned long long));
    if (err == cudaSuccess) err = cudaMalloc(&sv->lane_job, 2 * (size_t)ls->lanes * sizeof(pa::LaneJob));
    if (err == cudaSuccess)
        err = cudaMalloc(&sv->lane_stats, 2 * (size_t)ls->lanes * 4 * sizeof(unsigned long long));
    sv->stage_stride = 3 * ((size_t(1) << ls->cap) / 32 + 64);
    if (err == cudaSuccess) err = cudaMalloc(&sv->stage, (size_t)ls->lanes * sv->stage_stride * sizeof(uint32_t));
    if (err == cudaSuccess) err = cudaMemset(sv->claimed, 0, sizeof(unsigned long long));
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&sv->s, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&sv->ended, cudaEventDisableTiming);
    if (err != cudaSuccess) {
        free_serve(p);
        return cuda_fail(e, err);
    }
    std::memset(sv->ring, 0, sv->size * sizeof(pa::ServeSlot));
    std::memset(sv->ctl, 0, sizeof(pa::ServeCtl));
    sv->owner.assign(sv->size, ~0ull);
    sv->jobs.assign(sv->size, pa_job{});
    sv->geoms.assign(sv->size, BlockGeom{});
    rc = serve_launch(e, p);
    if (rc) {
        free_serve(p);
        return rc;
    }
    return ls->lanes;
}

int pa_serve_submit(pa_engine* e, const pa_job* job, uint64_t* ticket) {
    if (!e || !job || !ticket) return PA_ERR_INVALID_ARG;
    Pool* p = e->pool;
    if (!p || !p->serve) return PA_ERR_INVALID_ARG;
    ServeLoop* sv = p->serve;
    LaneSet* ls = p->lanes;
    PA_CUDA(e, cudaSetDevice(e->device));
    BlockGeom g, lg;
    int rc = job_geom(e, p, *job, &g);
    if (rc) return rc;
    rc = lane_geom(job->n, job->v, job->flags, &lg);
    if (rc) return rc;
    if (lg.log_np > ls->cap) return PA_ERR_TOO_LARGE;
    if (reinterpret_cast<uintptr_t>(job->out) & 3u) return PA_ERR_INVALID_ARG;
    if (sv->failed) {
        e->last_cuda = (int)cudaErrorLaunchTimeout;
        return PA_ERR_CUDA;
    }
    const uint32_t k = (uint32_t)(sv->next_ticket % sv->size);
    if (sv->owner[k] != ~0ull) return PA_ERR_BUSY;  // the ring is full: collect with pa_serve_poll
    pa::LaneJob j{};
    const void *ks = nullptr, *kr = nullptr, *sd = nullptr, *out = nullptr;
    if (!device_view(job->key_start, &ks) || !device_view(job->out, &out)) return PA_ERR_INVALID_ARG;
    if ((job->flags & PA_FLAG_XOR_KEY_REST) && !device_view(job->key_rest, &kr)) return PA_ERR_INVALID_ARG;
    j.key_start = static_cast<const uint32_t*>(ks);
    j.key_rest = static_cast<const uint32_t*>(kr);
    if (job->seed_id >= 0) {
        auto it = ls->spectra.find(lane_spec_key(job->seed_id, lg));
        if (it == ls->spectra.end()) return PA_ERR_NO_SEED;  // cache the seed before pa_serve_start
        j.spec = it->second.spec;
        j.seed_cnt = it->second.cnt + 1;
    } else {
        if (!device_view(job->seed_words, &sd)) return PA_ERR_INVALID_ARG;
        j.seed = static_cast<const uint32_t*>(sd);
    }
    j.out = static_cast<uint32_t*>(const_cast<void*>(out));
    j.g = lg;
    j.flags = job->flags;
    pa::ServeSlot* slot = sv->ring + k;
    slot->job = j;
    slot->err = 0;
    __atomic_store_n(&slot->done, 0ull, __ATOMIC_RELAXED);
    sv->owner[k] = sv->next_ticket;
    sv->jobs[k] = *job;
    sv->geoms[k] = g;
    *ticket = sv->next_ticket++;
    __atomic_store_n(&sv->ctl->tail, sv->next_ticket, __ATOMIC_RELEASE);  // publish
    if (!serve_running(sv)) {  // the loop ended (idle): start it again
        rc = serve_launch(e, p);
        if (rc) return rc;
    }
    return PA_OK;
}

int pa_serve_poll(pa_engine* e, uint64_t ticket, pa_stats* stats) {
    if (!e) return PA_ERR_INVALID_ARG;
    Pool* p = e->pool;
    if (!p || !p->serve) return PA_ERR_INVALID_ARG;
    ServeLoop* sv = p->serve;
    const uint32_t k = (uint32_t)(ticket % sv->size);
    if (sv->owner[k] != ticket) return PA_ERR_INVALID_ARG;
    pa::ServeSlot* slot = sv->ring + k;
    if (__atomic_load_n(&slot->done, __ATOMIC_ACQUIRE) != ticket + 1ull) {
        if (serve_running(sv)) return PA_PENDING;
        PA_CUDA(e, cudaSetDevice(e->device));
        cudaError_t q = cudaEventQuery(sv->ended);
        if (q != cudaSuccess && q != cudaErrorNotReady) return cuda_fail(e, q);
        if (__atomic_load_n(&slot->done, __ATOMIC_ACQUIRE) == ticket + 1ull) return PA_PENDING;  // just finished
        // the loop has ended without completing this request: a lane error, or a request it took and did
        // not finish, means the request is lost; otherwise it was published after the loop ended idle
        bool bad = false;
        int rc = serve_lane_error(e, p, &bad);
        if (rc) return rc;
        unsigned long long claimed = 0;
        PA_CUDA(e, cudaMemcpy(&claimed, sv->claimed, sizeof(claimed), cudaMemcpyDeviceToHost));
        if (bad || sv->failed || ticket < claimed) {
            sv->failed = true;
            sv->owner[k] = ~0ull;
            e->last_cuda = (int)cudaErrorLaunchTimeout;
            return PA_ERR_CUDA;
        }
        rc = serve_launch(e, p);
        return rc ? rc : PA_PENDING;
    }
    if (slot->err) {
        sv->owner[k] = ~0ull;
        e->last_cuda = (int)cudaErrorLaunchTimeout;
        return PA_ERR_CUDA;
    }
    float r;
    std::memcpy(&r, &slot->resid, sizeof(r));
    int exact = 0;
    if (!(r <= e->residual_limit)) {  // FP32 budget exceeded: recompute exactly from the host inputs
        PA_CUDA(e, cudaSetDevice(e->device));
        const pa_job& jb = sv->jobs[k];
        const BlockGeom& g = sv->geoms[k];
        Slot* sl = nullptr;
        int rc = exact_slot(e, p, g.log_np, &sl);
        if (rc) return rc;
        const uint32_t* seed = jb.seed_id >= 0 ? p->seeds[jb.seed_id].seed : sl->seed;
        if (jb.seed_id < 0)
            PA_CUDA(e, cudaMemcpyAsync(sl->seed, jb.seed_words, (size_t)(jb.n / 32u) * 4u, cudaMemcpyHostToDevice,
                                       sl->s));
        PA_CUDA(e, cudaMemcpyAsync(sl->ks, jb.key_start, (size_t)(g.h / 32u + 1u) * 4u, cudaMemcpyHostToDevice, sl->s));
        if (jb.flags & PA_FLAG_XOR_KEY_REST)
            PA_CUDA(e, cudaMemcpyAsync(sl->kr, jb.key_rest, (size_t)(jb.v / 32u) * 4u, cudaMemcpyHostToDevice, sl->s));
        rc = exact_in_slot(e, sl, g, seed, sl->ks, sl->kr, jb.flags, sl->out, sl->s);
        if (rc) return rc;
        PA_CUDA(e, cudaMemcpyAsync(jb.out, sl->out, pa_output_bytes(jb.n, jb.v, jb.flags), cudaMemcpyDeviceToHost,
                                   sl->s));
        PA_CUDA(e, cudaStreamSynchronize(sl->s));
        exact = 1;
    }
    if (stats) {
        stats->max_residual = r;
        stats->popcount_key = slot->cnt[0];
        stats->popcount_seed = slot->cnt[1];
        stats->gpu_ms = 0.f;
        stats->seed_uses_left = -1;
        stats->exact = exact;
    }
    sv->owner[k] = ~0ull;
    return PA_OK;
}

int pa_serve_stop(pa_engine* e) {
    if (!e) return PA_ERR_INVALID_ARG;
    Pool* p = e->pool;
    if (!p || !p->serve) return PA_OK;
    PA_CUDA(e, cudaSetDevice(e->device));
    free_serve(p);
    return PA_OK;
}

int pa_set_split(pa_engine* e, uint32_t log_n, uint32_t log_n2) {
    if (!e || log_n < 15 || log_n > 26) return PA_ERR_INVALID_ARG;
    if ((int)log_n2 < split_min((int)log_n) || (int)log_n2 > split_max((int)log_n)) return PA_ERR_INVALID_ARG;
    e->split[log_n] = (int8_t)log_n2;
    e->spec_valid = false;  // the cached single-block spectrum may use the old layout
    if (e->pool) drop_graphs(e->pool);
    return PA_OK;
}

int pa_get_split(pa_engine* e, uint32_t log_n) {
    if (!e || log_n < 15 || log_n > 26) return 0;
    int l2 = e->split[log_n];
    if (l2 < split_min((int)log_n) || l2 > split_max((int)log_n)) l2 = split_default((int)log_n);
    return l2;
}

int pa_autotune(pa_engine* e, uint32_t min_n, uint32_t max_n, float* ms_out) {
    if (!e || min_n < 1024u || max_n < min_n) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    Pool* p = get_pool(e);
    if (!p) return PA_ERR_CUDA;
    if (any_busy(p) || p->batch_pending) return PA_ERR_BUSY;
    const int lo = std::max(15, ceil_log2(min_n) - 1), hi = std::min(26, ceil_log2(max_n) - 1);
    if (ms_out)
        for (int i = 0; i < 32; ++i) ms_out[i] = 0.f;
    if (lo > hi) return PA_OK;
    // one slot of the largest size times every candidate
    const int cap = hi + 1;
    Slot* sl = nullptr;
    for (Slot* c : p->slots)
        if (!c->busy && c->cap >= cap && (!sl || c->cap < sl->cap)) sl = c;
    if (!sl) {
        if (!make_room(p, slot_bytes(cap))) return PA_ERR_TOO_LARGE;
        int rc = new_slot(e, p, cap, &sl);
        if (rc) return rc;
        p->slots.push_back(sl);
    }
    cudaStream_t s = sl->s;
    const size_t words = (size_t(1) << cap) / 32;
    PA_CUDA(e, cudaMemsetAsync(sl->seed, 0x5A, words * 4, s));  // data-independent timing: a fixed pattern
    PA_CUDA(e, cudaMemsetAsync(sl->ks, 0xA5, words * 4, s));
    PA_CUDA(e, cudaMemsetAsync(sl->kr, 0x3C, words * 4, s));
    cudaEvent_t t0, t1;
    PA_CUDA(e, cudaEventCreate(&t0));
    PA_CUDA(e, cudaEventCreate(&t1));
    int rc = PA_OK;
    for (int ln = lo; ln <= hi && !rc; ++ln) {
        const uint32_t n = 1u << (ln + 1), v = n / 4u + n / 8u;
        float best = 0.f;
        int best_l2 = split_default(ln);
        for (int l2 = split_min(ln); l2 <= split_max(ln) && !rc; ++l2) {
            int8_t tbl[32] = {};
            tbl[ln] = (int8_t)l2;
            BlockGeom g;
            rc = make_geom(n, v, PA_FLAG_XOR_KEY_REST | PA_FLAG_COMPRESS, tbl, &g);
            if (rc) break;
            rc = seed_in_slot(e, sl, g, sl->seed, sl->spec, sl->cnt + 1, s);
            float acc = 0.f;
            const int reps = 3;
            for (int r = 0; r <= reps && !rc; ++r) {  // first run warms up
                if (cudaEventRecord(t0, s) != cudaSuccess) rc = PA_ERR_CUDA;
                if (!rc) rc = key_in_slot(e, sl, g, sl->ks, sl->kr, PA_FLAG_XOR_KEY_REST | PA_FLAG_COMPRESS, sl->spec,
                                          sl->cnt, sl->resid, sl->out, s);
                if (!rc && cudaEventRecord(t1, s) != cudaSuccess) rc = PA_ERR_CUDA;
                if (!rc && cudaEventSynchronize(t1) != cudaSuccess) rc = PA_ERR_CUDA;
                float ms = 0.f;
                if (!rc) cudaEventElapsedTime(&ms, t0, t1);
                if (r) acc += ms;
            }
            if (rc) break;
            const float ms = acc / reps;
            if (best == 0.f || ms < best) {
                best = ms;
                best_l2 = l2;
            }
        }
        if (!rc) {
            e->split[ln] = (int8_t)best_l2;
            if (ms_out) ms_out[ln] = best;
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    int derr = 0;
    if (cudaMemcpy(&derr, sl->err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && derr) {
        cudaMemset(sl->err, 0, sizeof(int));
        e->last_cuda = (int)cudaErrorLaunchTimeout;
        rc = PA_ERR_CUDA;
    }
    e->spec_valid = false;
    drop_graphs(p);
    return rc;
}

}  // extern "C"
