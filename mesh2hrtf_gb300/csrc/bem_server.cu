// bem_server.cu - bem_server_*: solve requests served with continuous
// batching on one device.
//
// One worker thread per server owns two streams and a Krylov engine:
//  - admission: requests leave the queue in arrival order when an iteration
//    slot is free and their footprint fits the free part of the budget (a
//    first-fit arena over one device allocation made at creation, so admission
//    and release never call cudaMalloc/cudaFree);
//  - preparation on the second stream: frequency data, assembly (one
//    persistent launch for the admitted group), right-hand sides, block
//    inverses; it runs while the engine replays iteration bodies for the
//    requests already iterating;
//  - prepared requests join the engine's batch between two bodies, finished
//    ones leave it; their projection and result copies run on the second
//    stream and their memory returns to the arena.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "bem_solver.h"

namespace {

using Clock = std::chrono::steady_clock;
double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// First-fit allocator over [0, cap) with coalescing; host bookkeeping only.
class Arena {
public:
    explicit Arena(size_t cap) { free_[0] = cap; }
    bool alloc(size_t bytes, size_t *off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t o = it->first, rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[o + bytes] = rest;
            *off = o;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }

private:
    std::map<size_t, size_t> free_;
};

struct Request {
    uint64_t id = 0;
    bem_mesh_t mesh = nullptr;
    bem_frequency_desc fd{};
    std::vector<int32_t> bct;
    std::vector<double> bcv, adm, pxyz, pamp, pdir, pwamp, pts;
    int npts = 0;
    std::vector<double> x, pot, grad;
    bem_status rc = BEM_OK;
    std::string msg;
    bem_request_info info{};
    Clock::time_point t_submit, t_admit, t_join;
    bool done = false;
    size_t off = 0, bytes = 0, solver_bytes = 0;
    std::unique_ptr<bem_solver_s> solver;
};
using ReqP = std::shared_ptr<Request>;

// A group of admitted requests in preparation on the second stream.
struct Group {
    std::vector<ReqP> reqs;
    std::vector<int> slot;   // per request: its two status words in the pinned pool
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

size_t point_bytes(int npts) {
    return bem::round_up((size_t)npts * 24, 256) + bem::round_up((size_t)npts * 16, 256) +
           bem::round_up((size_t)npts * 48, 256);
}

}  // namespace

struct bem_server_s {
    bem_server_params prm{};
    int prec01 = 1;   // 0 complex128, 1 complex64
    int m = 60;
    unsigned char *base = nullptr;
    size_t cap = 0;
    std::unique_ptr<Arena> arena;   // guarded by mu
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ReqP> pending;
    std::map<uint64_t, ReqP> live;
    uint64_t next_id = 1;
    bool stop = false;
    std::thread worker;

    void finish(const ReqP &r, bem_status rc, const std::string &msg) {
        r->solver.reset();
        std::lock_guard<std::mutex> lk(mu);
        r->rc = rc;
        r->msg = msg;
        r->info.latency_ms = ms_between(r->t_submit, Clock::now());
        arena->release(r->off, r->bytes);
        r->done = true;
        cv_done.notify_all();
        cv_work.notify_all();
    }
    void run();
};

namespace {

std::string last_msg() { return bem_last_error(); }

// Solver over the request's arena block, frequency data uploaded on st.
bem_status make_solver(bem_server_s *S, const ReqP &r, cudaStream_t st) {
    std::unique_ptr<bem_solver_s> s(new bem_solver_s());
    const int n = r->mesh->n;
    s->mesh = r->mesh;
    s->n = n;
    s->prec = S->prm.precision;
    s->restart = S->m;
    s->max_iter = S->prm.max_iter > 0 ? S->prm.max_iter : 1000;
    s->tol = S->prm.tol > 0 ? S->prm.tol : 1e-9;
    s->lda = bem::round_up((size_t)n, 32);
    s->precond = true;
    s->own_block = false;
    s->block = S->base + r->off;
    s->block_bytes = r->solver_bytes;
    bem::solver_layout(n, S->prec01, S->m, true, s->block, &s->d);
    unsigned char *p = s->block + r->solver_bytes;
    s->pts = (double *)p;
    p += bem::round_up((size_t)r->npts * 24, 256);
    s->pot = (double *)p;
    p += bem::round_up((size_t)r->npts * 16, 256);
    s->grad = (double *)p;
    s->pts_cap = r->npts;
    r->solver = std::move(s);
    return bem::upload_freq(r->solver.get(), &r->fd, st);
}

}  // namespace

void bem_server_s::run() {
    cudaSetDevice(prm.device);
    cudaStream_t st_k = nullptr, st_a = nullptr;
    cudaStreamCreateWithFlags(&st_k, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&st_a, cudaStreamNonBlocking);
    unsigned *ctr = nullptr;
    cudaMalloc(&ctr, 4 * sizeof(unsigned));
    // pinned status words of the requests in preparation (assembly, block
    // inverse): at most max_active requests are in preparation at once
    int *h_pool = nullptr;
    cudaMallocHost(&h_pool, 2 * sizeof(int) * bem::kMaxSys);
    std::vector<int> free_slots;
    for (int i = bem::kMaxSys - 1; i >= 0; --i) free_slots.push_back(i);
    cudaMemset(ctr, 0, 4 * sizeof(unsigned));
    cudaEvent_t pe0 = nullptr, pe1 = nullptr;
    cudaEventCreate(&pe0);
    cudaEventCreate(&pe1);
    std::unique_ptr<bem::Engine> eng(new bem::Engine(prec01, st_k));
    std::vector<ReqP> active;
    std::vector<bem::KState> states;
    std::deque<Group> prep;
    bool changed = false;
    int n_prep = 0;
    auto fail_all = [&](const std::string &msg) {
        for (auto &r : active) finish(r, BEM_ERR_CUDA, msg);
        active.clear();
        states.clear();
    };
    while (true) {
        // ---- admission (arrival order; head of line waits for memory)
        std::vector<ReqP> adm;
        {
            std::unique_lock<std::mutex> lk(mu);
            int slots = prm.max_active - (int)active.size() - n_prep;
            while (slots > 0 && !pending.empty()) {
                ReqP r = pending.front();
                size_t off = 0;
                if (!arena->alloc(r->bytes, &off)) break;
                r->off = off;
                r->t_admit = Clock::now();
                r->info.queued_ms = ms_between(r->t_submit, r->t_admit);
                pending.pop_front();
                adm.push_back(r);
                --slots;
            }
            if (adm.empty() && active.empty() && prep.empty()) {
                if (stop) break;
                cv_work.wait(lk, [&] { return stop || !pending.empty(); });
                continue;
            }
        }
        // ---- preparation of the admitted group on the second stream
        if (!adm.empty()) {
            Group g;
            std::vector<bem_solver_t> ss;
            for (auto &r : adm) {
                bem_status rc = make_solver(this, r, st_a);
                if (rc != BEM_OK) finish(r, rc, last_msg());
                else g.reqs.push_back(r);
            }
            for (auto &r : g.reqs) ss.push_back(r->solver.get());
            if (!ss.empty()) {
                cudaEventCreate(&g.e0);
                cudaEventCreate(&g.e1);
                for (size_t i = 0; i < ss.size(); ++i) {
                    g.slot.push_back(free_slots.back());
                    free_slots.pop_back();
                }
                const int cnt = (int)ss.size();
                cudaEventRecord(g.e0, st_a);
                std::unique_ptr<bem::AsmBatch> at(new bem::AsmBatch());
                std::unique_ptr<bem::PcBatch> pt(new bem::PcBatch());
                cudaError_t e = cudaSuccess;
                for (int i = 0; i < cnt; ++i) {
                    if (e == cudaSuccess) e = cudaMemsetAsync(ss[i]->d.status, 0, sizeof(int), st_a);
                    if (e == cudaSuccess) e = cudaMemsetAsync(ss[i]->d.x, 0, sizeof(double2) * ss[i]->n, st_a);
                }
                // launch shapes the tuner chose earlier for these sizes (the
                // serving loop looks them up; it does not tune)
                int big = 0;
                for (int i = 1; i < cnt; ++i)
                    if (ss[i]->n > ss[big]->n) big = i;
                const bem::AsmShape shape = bem::tune_lookup(ss[big]->n, ss[big]->prec, 1).asm_shape;
                for (int i = 0; i < cnt; ++i) ss[i]->mv_strip = bem::tune_lookup(ss[i]->n, ss[i]->prec, 1).mv_strip;
                for (int c0 = 0; c0 < cnt && e == cudaSuccess; c0 += bem::kMaxAsm) {
                    const int k = std::min(bem::kMaxAsm, cnt - c0);
                    at->B = k;
                    for (int i = 0; i < k; ++i) at->sys[i] = ss[c0 + i]->asys();
                    bem::asm_batch_finish(*at);
                    e = bem::launch_assemble(*at, prec01, ctr, st_a, shape);
                    if (e == cudaSuccess) e = bem::launch_rhs(*at, st_a);
                }
                for (int i = 0; i < cnt && e == cudaSuccess; ++i) {
                    e = cudaMemcpyAsync(&h_pool[2 * g.slot[i]], ss[i]->d.status, sizeof(int), cudaMemcpyDeviceToHost,
                                        st_a);
                    if (e == cudaSuccess) e = cudaMemsetAsync(ss[i]->d.status, 0, sizeof(int), st_a);
                }
                for (int c0 = 0; c0 < cnt && e == cudaSuccess; c0 += bem::kMaxAsm) {
                    const int k = std::min(bem::kMaxAsm, cnt - c0);
                    pt->B = k;
                    for (int i = 0; i < k; ++i) pt->sys[i] = ss[c0 + i]->psys();
                    bem::pc_batch_finish(*pt);
                    e = bem::launch_block_inverse(*pt, prec01, st_a);
                }
                if (e == cudaSuccess) e = bem::split_group(ss.data(), cnt, st_a);
                for (int i = 0; i < cnt && e == cudaSuccess; ++i)
                    e = cudaMemcpyAsync(&h_pool[2 * g.slot[i] + 1], ss[i]->d.status, sizeof(int),
                                        cudaMemcpyDeviceToHost, st_a);
                if (e == cudaSuccess) e = cudaEventRecord(g.e1, st_a);
                if (e != cudaSuccess) {
                    cudaStreamSynchronize(st_a);
                    for (auto &r : g.reqs) finish(r, BEM_ERR_CUDA, cudaGetErrorString(e));
                    for (int sl : g.slot) free_slots.push_back(sl);
                    cudaEventDestroy(g.e0);
                    cudaEventDestroy(g.e1);
                } else {
                    n_prep += cnt;
                    prep.push_back(g);
                }
            }
        }
        // ---- prepared groups join the batch
        while (!prep.empty() && cudaEventQuery(prep.front().e1) == cudaSuccess) {
            Group g = prep.front();
            prep.pop_front();
            n_prep -= (int)g.reqs.size();
            float ams = 0.f;
            cudaEventElapsedTime(&ams, g.e0, g.e1);
            for (size_t i = 0; i < g.reqs.size(); ++i) {
                ReqP r = g.reqs[i];
                bem_solver_t s = r->solver.get();
                const int asm_st = h_pool[2 * g.slot[i]], pc_st = h_pool[2 * g.slot[i] + 1];
                free_slots.push_back(g.slot[i]);
                s->info.assemble_ms = ams;
                s->info.n_near_pairs = (int64_t)(s->mesh->n_near - s->n);
                if (asm_st != 0) {
                    finish(r, BEM_ERR_SUBDIVISION,
                           asm_st == 1 ? "number of subelements which are subdivided in a loop must <= 15"
                                       : "number of subelements must be < 220");
                    continue;
                }
                s->have_precond = pc_st == 0;
                s->have_freq = true;
                s->factored = false;
                r->t_join = Clock::now();
                active.push_back(r);
                states.push_back(s->kinit());
                changed = true;
            }
            cudaEventDestroy(g.e0);
            cudaEventDestroy(g.e1);
        }
        if (active.empty()) {
            if (!prep.empty()) cudaEventSynchronize(prep.front().e1);
            continue;
        }
        // ---- one iteration body for every request in the batch
        if (changed) {
            std::vector<bem::KSys> sys;
            for (auto &r : active) sys.push_back(r->solver->ksys());
            cudaError_t e = eng->set_batch(sys, states);
            if (e != cudaSuccess) {
                fail_all(cudaGetErrorString(e));
                continue;
            }
            changed = false;
        }
        cudaError_t be = eng->run_body();
        if (be != cudaSuccess) {
            fail_all(be == cudaErrorLaunchTimeout ? "matrix-vector product: a bounded device wait gave up"
                                                  : cudaGetErrorString(be));
            continue;
        }
        std::vector<ReqP> fin;
        std::vector<ReqP> keep;
        std::vector<bem::KState> keep_st;
        for (size_t i = 0; i < active.size(); ++i) {
            const bem::KState &q = eng->states()[i];
            if (q.phase == bem::kPhaseFinished) {
                bem_solver_t s = active[i]->solver.get();
                s->info.iterations = q.iters;
                s->info.restarts = q.cycles;
                s->info.rel_residual = q.rel;
                s->info.n_matvec = q.n_mv;
                s->info.solve_ms = ms_between(active[i]->t_join, Clock::now());
                s->info.matvec_ms = 0.0;
                s->solved = true;
                fin.push_back(active[i]);
            } else {
                keep.push_back(active[i]);
                keep_st.push_back(q);
            }
        }
        if (fin.empty()) {
            for (size_t i = 0; i < active.size(); ++i) states[i] = eng->states()[i];
            continue;
        }
        // states of the finished requests, for their statuses
        std::vector<bem::KState> fin_st;
        for (size_t i = 0; i < active.size(); ++i)
            if (eng->states()[i].phase == bem::kPhaseFinished) fin_st.push_back(eng->states()[i]);
        active.swap(keep);
        states.swap(keep_st);
        changed = true;
        // ---- projection and results of the finished requests
        std::vector<bem_solver_t> ss;
        std::vector<int32_t> np;
        std::vector<const double *> pp;
        std::vector<double *> po, pg;
        for (auto &r : fin) {
            r->x.assign(2 * (size_t)r->mesh->n, 0.0);
            r->pot.assign(2 * (size_t)r->npts, 0.0);
            r->grad.assign(6 * (size_t)r->npts, 0.0);
            ss.push_back(r->solver.get());
            np.push_back(r->npts);
            pp.push_back(r->npts ? r->pts.data() : nullptr);
            po.push_back(r->npts ? r->pot.data() : nullptr);
            pg.push_back(r->npts ? r->grad.data() : nullptr);
        }
        std::vector<bem_status> prc(fin.size(), BEM_OK);
        bem_status grc = bem::project_group(ss.data(), (int)ss.size(), np.data(), pp.data(), po.data(), pg.data(),
                                            st_a, pe0, pe1, prc.data());
        std::string gmsg = grc != BEM_OK ? last_msg() : std::string();
        for (size_t i = 0; i < fin.size(); ++i) {
            ReqP r = fin[i];
            bem_solver_t s = r->solver.get();
            bem_status rc = grc == BEM_ERR_CUDA ? grc : prc[i];
            std::string msg = rc != BEM_OK ? gmsg : std::string();
            if (rc == BEM_OK) {
                rc = bem::solution_to_host(s, st_a, r->x.data());
                if (rc != BEM_OK) msg = last_msg();
            }
            if (rc == BEM_OK) {
                rc = bem::map_result(fin_st[i]);
                if (rc != BEM_OK) msg = last_msg();
            }
            r->info.solve = s->info;
            finish(r, rc, msg);
        }
    }
    for (auto &g : prep) {
        cudaEventDestroy(g.e0);
        cudaEventDestroy(g.e1);
    }
    eng.reset();
    cudaFreeHost(h_pool);
    cudaEventDestroy(pe0);
    cudaEventDestroy(pe1);
    cudaFree(ctr);
    cudaStreamDestroy(st_k);
    cudaStreamDestroy(st_a);
}

extern "C" {

bem_status bem_server_create(const bem_server_params *p, bem_server_t *out) {
    if (!p || !out) return bem::fail(BEM_ERR_INVALID, "null argument");
    *out = nullptr;
    if (p->precision != BEM_PREC_FP64 && p->precision != BEM_PREC_MIXED)
        return bem::fail(BEM_ERR_INVALID, "unknown precision %d", p->precision);
    const int m = p->restart > 0 ? p->restart : 60;
    if (m > bem::kMaxRestart) return bem::fail(BEM_ERR_INVALID, "restart length %d above the limit %d", m, bem::kMaxRestart);
    if (p->max_active < 0 || p->max_active > bem::kMaxSys)
        return bem::fail(BEM_ERR_INVALID, "max_active %d outside 0..%d", p->max_active, bem::kMaxSys);
    bem_status rc = bem_set_device(p->device);
    if (rc != BEM_OK) return rc;
    std::unique_ptr<bem_server_s> S(new bem_server_s());
    S->prm = *p;
    if (S->prm.max_active == 0) S->prm.max_active = bem::kMaxSys;
    S->prec01 = p->precision == BEM_PREC_FP64 ? 0 : 1;
    S->m = m;
    size_t free_b = 0, total_b = 0;
    BEM_CU(cudaMemGetInfo(&free_b, &total_b));
    // the arena is one block: hand the library's cached blocks back first
    bem::dev_release_cached(p->device);
    BEM_CU(cudaMemGetInfo(&free_b, &total_b));
    double budget = p->hbm_budget_bytes > 0 ? p->hbm_budget_bytes : (double)free_b - 1.0e9;
    if (budget <= 0 || budget > (double)free_b)
        return bem::fail(BEM_ERR_OUT_OF_HBM, "server budget %.3f GB, device has %.3f GB free", budget / 1e9,
                         free_b / 1e9);
    S->cap = bem::round_up((size_t)budget, 256) - 256;
    cudaError_t e = cudaMalloc(&S->base, S->cap);
    if (e != cudaSuccess)
        return bem::fail(e == cudaErrorMemoryAllocation ? BEM_ERR_OUT_OF_HBM : BEM_ERR_CUDA, "server budget: %s",
                         cudaGetErrorString(e));
    S->arena.reset(new Arena(S->cap));
    bem_server_s *raw = S.get();
    S->worker = std::thread([raw] { raw->run(); });
    *out = S.release();
    return BEM_OK;
}

bem_status bem_server_submit(bem_server_t S, bem_mesh_t mesh, const bem_frequency_desc *f, int32_t n_pts,
                             const double *pts, uint64_t *ticket) {
    if (!S || !mesh || !f || !ticket) return bem::fail(BEM_ERR_INVALID, "null argument");
    if (n_pts < 0 || (n_pts > 0 && !pts)) return bem::fail(BEM_ERR_INVALID, "bad point arrays");
    if (!(f->wave_number > 0.0)) return bem::fail(BEM_ERR_INVALID, "wave number must be > 0");
    if (f->n_point < 0 || f->n_plane < 0 || (f->n_point && (!f->point_xyz || !f->point_amp)) ||
        (f->n_plane && (!f->plane_dir || !f->plane_amp)))
        return bem::fail(BEM_ERR_INVALID, "source arrays missing");
    auto r = std::make_shared<Request>();
    const int n = mesh->n;
    r->mesh = mesh;
    r->fd = *f;
    if (f->bc_type) r->bct.assign(f->bc_type, f->bc_type + n);
    if (f->bc_value) r->bcv.assign(f->bc_value, f->bc_value + 8 * (size_t)n);
    if (f->admittance) r->adm.assign(f->admittance, f->admittance + 2 * (size_t)n);
    if (f->n_point) {
        r->pxyz.assign(f->point_xyz, f->point_xyz + 3 * (size_t)f->n_point);
        r->pamp.assign(f->point_amp, f->point_amp + 2 * (size_t)f->n_point);
    }
    if (f->n_plane) {
        r->pdir.assign(f->plane_dir, f->plane_dir + 3 * (size_t)f->n_plane);
        r->pwamp.assign(f->plane_amp, f->plane_amp + 2 * (size_t)f->n_plane);
    }
    r->fd.bc_type = f->bc_type ? r->bct.data() : nullptr;
    r->fd.bc_value = f->bc_value ? r->bcv.data() : nullptr;
    r->fd.admittance = f->admittance ? r->adm.data() : nullptr;
    r->fd.point_xyz = r->pxyz.data();
    r->fd.point_amp = r->pamp.data();
    r->fd.plane_dir = r->pdir.data();
    r->fd.plane_amp = r->pwamp.data();
    r->npts = n_pts;
    if (n_pts) r->pts.assign(pts, pts + 3 * (size_t)n_pts);
    r->solver_bytes = bem::solver_layout(n, S->prec01, S->m, true, nullptr, nullptr);
    r->bytes = r->solver_bytes + point_bytes(n_pts);
    if (r->bytes > S->cap)
        return bem::fail(BEM_ERR_OUT_OF_HBM, "request for %d unknowns needs %.3f GB, server budget %.3f GB", n,
                         r->bytes / 1e9, S->cap / 1e9);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) return bem::fail(BEM_ERR_INVALID, "server is stopping");
        r->id = S->next_id++;
        S->live[r->id] = r;
        S->pending.push_back(r);
    }
    S->cv_work.notify_all();
    *ticket = r->id;
    return BEM_OK;
}

bem_status bem_server_wait(bem_server_t S, uint64_t ticket, double timeout_s, double *x_out, double *pot_out,
                           double *grad_out, bem_request_info *info) {
    if (!S) return bem::fail(BEM_ERR_INVALID, "null server");
    ReqP r;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->live.find(ticket);
        if (it == S->live.end()) return bem::fail(BEM_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
        r = it->second;
        auto ready = [&] { return r->done; };
        if (timeout_s < 0) S->cv_done.wait(lk, ready);
        else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
            return bem::fail(BEM_ERR_PENDING, "request %llu not finished", (unsigned long long)ticket);
        S->live.erase(it);
    }
    if (x_out && !r->x.empty()) std::memcpy(x_out, r->x.data(), sizeof(double) * r->x.size());
    if (pot_out && !r->pot.empty()) std::memcpy(pot_out, r->pot.data(), sizeof(double) * r->pot.size());
    if (grad_out && !r->grad.empty()) std::memcpy(grad_out, r->grad.data(), sizeof(double) * r->grad.size());
    if (info) *info = r->info;
    if (r->rc != BEM_OK) return bem::fail(r->rc, "%s", r->msg.c_str());
    return BEM_OK;
}

bem_status bem_server_destroy(bem_server_t S) {
    if (!S) return BEM_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        for (auto &r : S->pending) {
            r->rc = BEM_ERR_INVALID;
            r->msg = "server stopped before the request was admitted";
            r->done = true;
        }
        S->pending.clear();
    }
    S->cv_work.notify_all();
    S->cv_done.notify_all();
    if (S->worker.joinable()) S->worker.join();
    cudaFree(S->base);
    delete S;
    return BEM_OK;
}

}  // extern "C"
