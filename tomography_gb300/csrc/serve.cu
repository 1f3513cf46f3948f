// Serving loop: continuous batching of candidate-evaluation requests.
//
// The reference farms candidates over MPI ranks, one blocking FDTD_GPU call
// per rank and candidate (test.cxx:82-121, tao master/worker).  Here one
// process keeps every admitted solve resident on the GPU:
//   * tomo_submit / tomo_submit_spec queue a request (n_cand candidates, each
//     n_exc solves; a request may carry its own grid spec);
//   * tomo_serve_step admits queued requests in FIFO order while their memory
//     fits the HBM budget and descriptor slots are free, then advances EVERY
//     admitted solve by up to four launches of the descriptor-driven advance
//     kernel (solves of different requests, grid sizes and progress share
//     the launches), and retires requests whose solves reached their last step
//     (far field + misfit on the device, fitness to the host);
//   * tomo_poll returns a finished request's fitness.
// Each solve's arithmetic depends only on its own descriptor, so a result is
// bit-identical whether the request ran alone or mixed with others.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "engine_impl.cuh"

namespace tomo {

constexpr int kServeSlots = 1 << 16;   // descriptor slots (solves in flight)

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2, kCancelled = 3, kFailed = 4 };

template <typename Real>
struct ServeRequest {
    uint64_t ticket = 0;
    ClassData<Real>* cd = nullptr;
    std::vector<double> args;
    size_t ncand = 0;
    int nsolves = 0, first = -1;
    int state = kQueued;
    int steps_done = 0;
    int status = TOMO_OK;
    Unpacked up;
    void* mem = nullptr;      // stream-ordered allocation holding everything below
    size_t bytes = 0;
    Real* state_base = nullptr;
    uint8_t* mats = nullptr;
    Real* tabs = nullptr;
    double* upload = nullptr;
    float* D = nullptr;
    float* P = nullptr;
    double* partials = nullptr;
    double* fit = nullptr;
    int* flag = nullptr;
    std::vector<double> fitness;
    int hflag = 0;
};

template <typename Real>
struct ServeStateT {
    DevBuf descs, items;
    std::vector<SolveDesc<Real>> hdescs;
    std::vector<char> used;
    std::map<uint64_t, std::unique_ptr<ServeRequest<Real>>> reqs;
    std::deque<uint64_t> queue;
    std::vector<std::unique_ptr<ClassData<Real>>> classes;
    uint64_t next_ticket = 1;
    uint64_t bytes_in_use = 0;
    bool items_dirty = false;
    int nitems = 0, blocks = 0;
    size_t smem = 0;
    int hi_slot = 0;   // one past the highest slot ever used
    Blocking blk{0, 0, 0};   // blocking of the serving loop, fixed at the first serving step
    int cmax = 0;             // largest NTFF contour among the running requests

    int find_range(int n) {
        int run = 0;
        for (int i = 0; i < kServeSlots; ++i) {
            run = used[i] ? 0 : run + 1;
            if (run == n) return i - n + 1;
        }
        return -1;
    }
};

template <typename Real>
static ServeStateT<Real>* serve_state(ServeStateT<Real>*& s, int* rc) {
    *rc = TOMO_OK;
    if (s) return s;
    auto* st = new ServeStateT<Real>();
    st->hdescs.assign(kServeSlots, SolveDesc<Real>{});
    st->used.assign(kServeSlots, 0);
    *rc = st->descs.ensure(sizeof(SolveDesc<Real>) * kServeSlots);
    if (*rc == TOMO_OK && cudaMemset(st->descs.p, 0, sizeof(SolveDesc<Real>) * kServeSlots) != cudaSuccess)
        *rc = fail(TOMO_ECUDA, "cudaMemset of serving descriptors failed");
    if (*rc) {
        delete st;
        return nullptr;
    }
    s = st;
    return s;
}

template <typename Real>
void EngineT<Real>::serve_release() {
    if (!serve_) return;
    cudaStreamSynchronize(stream_);
    for (auto& kv : serve_->reqs)
        if (kv.second->mem) cudaFree(kv.second->mem);
    delete serve_;
    serve_ = nullptr;
}

template <typename Real>
static int request_submit(EngineT<Real>* eng, ServeStateT<Real>* st, ClassData<Real>* cd, const double* args,
                          size_t ncand, size_t nparam, uint64_t* ticket) {
    if (!ticket) return fail(TOMO_EINVAL, "ticket is NULL");
    if (cd->pc.extra)
        return fail(TOMO_EINVAL, "the total-field variant runs through forward: the serving loop carries no incident grid");
    auto r = std::make_unique<ServeRequest<Real>>();
    TOMO_TRY(unpack_args(cd->pc, args, ncand, nparam, r->up));
    if (!cd->have_target) return fail(TOMO_ENOTARGET, "serving needs a target for this spec");
    r->ticket = st->next_ticket++;
    r->cd = cd;
    r->ncand = ncand;
    r->nsolves = (int)ncand * cd->pc.n_exc;
    if (r->nsolves > kServeSlots) return fail(TOMO_EINVAL, "request larger than the serving slot table");
    *ticket = r->ticket;
    st->queue.push_back(r->ticket);
    st->reqs[r->ticket] = std::move(r);
    (void)eng;
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::submit(const double* args, size_t ncand, size_t nparam, uint64_t* ticket) {
    int rc;
    ServeStateT<Real>* st = serve_state(serve_, &rc);
    if (!st) return rc;
    return request_submit(this, st, &cd_, args, ncand, nparam, ticket);
}

template <typename Real>
int EngineT<Real>::submit_spec(const tomo_spec* spec, const double* args, size_t ncand, size_t nparam,
                               uint64_t* ticket) {
    if (!spec) return submit(args, ncand, nparam, ticket);
    int rc;
    ServeStateT<Real>* st = serve_state(serve_, &rc);
    if (!st) return rc;
    ClassData<Real>* cd = class_for(spec, &rc);
    if (!cd) return rc;
    return request_submit(this, st, cd, args, ncand, nparam, ticket);
}

template <typename Real>
ClassData<Real>* EngineT<Real>::class_for(const tomo_spec* spec, int* rc) {
    *rc = TOMO_OK;
    if (!spec || same_problem(*spec, cd_.pc.spec)) return &cd_;
    if (spec->precision != cd_.pc.spec.precision || advance_mode(*spec) != advance_mode(cd_.pc.spec)) {
        *rc = fail(TOMO_EINVAL, "a handle serves one precision and one mode family");
        return nullptr;
    }
    ServeStateT<Real>* st = serve_state(serve_, rc);
    if (!st) return nullptr;
    for (auto& c : st->classes)
        if (same_problem(*spec, c->pc.spec)) return c.get();
    ProblemClass pc;
    if ((*rc = build_class(*spec, pc))) return nullptr;
    auto cd = std::make_unique<ClassData<Real>>();
    if ((*rc = cd->init(pc))) return nullptr;
    st->classes.push_back(std::move(cd));
    return st->classes.back().get();
}

template <typename Real>
int EngineT<Real>::set_target_spec(const tomo_spec* spec, const float* t, size_t n) {
    int rc;
    ClassData<Real>* cd = class_for(spec, &rc);
    if (!cd) return rc;
    return cd->set_target(t, n);
}

// Device memory of one request: state of every solve, material maps and
// tables, the argument upload, far field, misfit partials and fitness, in one
// stream-ordered allocation.
struct RequestLayout {
    size_t state, mats, tabs, up, ff, part, fit, total;
};

template <typename Real>
static RequestLayout request_layout(const ClassData<Real>& cd, size_t ncand, size_t upload_doubles) {
    const ProblemClass& pc = cd.pc;
    const SolveLayout& L = cd.lay;
    const size_t nsolves = ncand * (size_t)pc.n_exc;
    auto align = [](size_t v) { return (v + 255) / 256 * 256; };
    RequestLayout b{};
    b.state = align(sizeof(Real) * nsolves * L.per_solve);
    b.mats = pc.spec.mode == TOMO_MODE_BREAST ? align(L.mat_stride * ncand) : 0;
    b.tabs = align(sizeof(Real) * kMaxMat * kMatCoef * ncand);
    b.up = align(sizeof(double) * upload_doubles);
    // far field only where the misfit needs it (reference modes); a served
    // request returns its fitness alone
    b.ff = pc.nang > 0 && pc.spec.mode != TOMO_MODE_BREAST ? align(sizeof(float) * nsolves * pc.nfreq * pc.nang) : 0;
    b.part = align(sizeof(double) * 2 * nsolves);
    b.fit = align(sizeof(double) * ncand);
    b.total = b.state + b.mats + b.tabs + b.up + 2 * b.ff + b.part + b.fit + 256;
    return b;
}

// doubles of the packed argument upload of ncand candidates (unpack_args)
inline size_t upload_doubles(const ProblemClass& pc, size_t ncand) {
    const int K = pc.spec.mode == TOMO_MODE_BREAST ? pc.spec.n_ellipses : 0;
    return ncand * kMaxMat * 3 + ncand * (size_t)K * 6;
}

template <typename Real>
int EngineT<Real>::request_bytes(const tomo_spec* spec, size_t ncand, uint64_t* bytes) {
    if (ncand == 0) return fail(TOMO_EINVAL, "no candidates");
    int rc;
    ClassData<Real>* cd = class_for(spec, &rc);
    if (!cd) return rc;
    *bytes = request_layout(*cd, ncand, upload_doubles(cd->pc, ncand)).total;
    return TOMO_OK;
}

template <typename Real>
static int admit(EngineT<Real>* eng, ServeStateT<Real>* st, ServeRequest<Real>& r, cudaStream_t stream,
                 uint64_t budget, bool* admitted) {
    *admitted = false;
    const ClassData<Real>& cd = *r.cd;
    const RequestLayout lay = request_layout(cd, r.ncand, r.up.upload.size());
    const size_t b_state = lay.state, b_mats = lay.mats, b_tabs = lay.tabs, b_up = lay.up, b_ff = lay.ff,
                 b_part = lay.part, b_fit = lay.fit, bytes = lay.total;
    if (st->bytes_in_use + bytes > budget) {
        if (st->bytes_in_use == 0)
            return fail(TOMO_ENOMEM_BUDGET, "request needs " + std::to_string(bytes >> 20) + " MiB, above the budget");
        return TOMO_OK;   // wait for memory to free up
    }
    const int first = st->find_range(r.nsolves);
    if (first < 0) return TOMO_OK;   // wait for descriptor slots
    void* mem = nullptr;
    cudaError_t e = cudaMallocAsync(&mem, bytes, stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (st->bytes_in_use == 0) return fail(TOMO_ENOMEM_BUDGET, "device allocation failed for a single request");
        return TOMO_OK;
    }
    char* p = (char*)mem;
    r.mem = mem;
    r.bytes = bytes;
    r.state_base = (Real*)p; p += b_state;
    r.mats = b_mats ? (uint8_t*)p : nullptr; p += b_mats;
    r.tabs = (Real*)p; p += b_tabs;
    r.upload = (double*)p; p += b_up;
    r.D = b_ff ? (float*)p : nullptr; p += b_ff;
    r.P = b_ff ? (float*)p : nullptr; p += b_ff;
    r.partials = (double*)p; p += b_part;
    r.fit = (double*)p; p += b_fit;
    r.flag = (int*)p;
    // set-up of the admitted request; on any failure the allocation is
    // returned at once (it was never charged to the budget)
    auto setup = [&]() -> int {
        int64_t kernels = 0, h2d = 0;
        TOMO_TRY(setup_materials<Real>(cd, r.up, r.upload, r.mats, r.tabs, stream, &kernels, &h2d));
        CUDA_TRY(cudaMemsetAsync(r.state_base, 0, b_state, stream));
        CUDA_TRY(cudaMemsetAsync(r.flag, 0, sizeof(int), stream));
        fill_descs<Real>(cd, r.up, r.state_base, r.mats, r.tabs, &st->hdescs[first]);
        CUDA_TRY(cudaMemcpyAsync(st->descs.template as<SolveDesc<Real>>() + first, &st->hdescs[first],
                                 sizeof(SolveDesc<Real>) * r.nsolves, cudaMemcpyHostToDevice, stream));
        return TOMO_OK;
    };
    if (const int rc = setup()) {
        for (int i = 0; i < r.nsolves; ++i) st->hdescs[first + i] = SolveDesc<Real>{};
        cudaFreeAsync(r.mem, stream);
        r.mem = nullptr;
        r.bytes = 0;
        return rc;
    }
    for (int i = 0; i < r.nsolves; ++i) st->used[first + i] = 1;
    st->hi_slot = std::max(st->hi_slot, first + r.nsolves);
    st->bytes_in_use += bytes;
    r.first = first;
    r.state = kRunning;
    r.steps_done = 0;
    st->items_dirty = true;
    *admitted = true;
    (void)eng;
    return TOMO_OK;
}

template <typename Real>
static int retire(ServeStateT<Real>* st, ServeRequest<Real>& r, cudaStream_t stream, bool success) {
    if (success) {
        int64_t kernels = 0;
        TOMO_TRY(post_range<Real>(*r.cd, r.ncand, st->hdescs[r.first], true, r.D, r.P, r.partials, r.fit, r.flag,
                                  nullptr, nullptr, stream, &kernels));
        r.fitness.assign(r.ncand, 0.0);
        CUDA_TRY(cudaMemcpyAsync(r.fitness.data(), r.fit, sizeof(double) * r.ncand, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaMemcpyAsync(&r.hflag, r.flag, sizeof(int), cudaMemcpyDeviceToHost, stream));
    }
    // deactivate the descriptors (the bump kernel and the advance kernel skip them)
    for (int i = 0; i < r.nsolves; ++i) {
        st->hdescs[r.first + i] = SolveDesc<Real>{};
        st->used[r.first + i] = 0;
    }
    CUDA_TRY(cudaMemcpyAsync(st->descs.template as<SolveDesc<Real>>() + r.first, &st->hdescs[r.first],
                             sizeof(SolveDesc<Real>) * r.nsolves, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaFreeAsync(r.mem, stream));
    st->bytes_in_use -= r.bytes;
    r.mem = nullptr;
    st->items_dirty = true;
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::serve_step(int* n_active) {
    int rc;
    ServeStateT<Real>* st = serve_state(serve_, &rc);
    if (!st) return rc;
    if (st->blk.T == 0) st->blk = blk_;   // the blocking stays fixed while requests are in flight
    // 1. admit queued requests in arrival order
    while (!st->queue.empty()) {
        auto it = st->reqs.find(st->queue.front());
        if (it == st->reqs.end() || it->second->state != kQueued) {
            st->queue.pop_front();
            continue;
        }
        bool admitted = false;
        rc = admit(this, st, *it->second, stream_, budget_, &admitted);
        if (rc) {
            it->second->state = kFailed;
            it->second->status = rc;
            st->queue.pop_front();
            return rc;
        }
        if (!admitted) break;
        st->queue.pop_front();
    }
    // 2. work items of every running solve
    if (st->items_dirty) {
        std::vector<WorkItem> items;
        long strips = 0;
        int nymax = 0;
        for (auto& kv : st->reqs) {
            const ServeRequest<Real>& r = *kv.second;
            if (r.state != kRunning) continue;
            const ProblemClass& pc = r.cd->pc;
            strips += (long)r.nsolves * items_per_solve(pc.nx, pc.ny, pc.nc, item_face_distance(pc), st->blk.T,
                                                       st->blk.cols);
            nymax = std::max(nymax, pc.ny);
        }
        const int nseg = choose_segments(strips, nymax, st->blk.T, 24L * num_sms_);
        st->cmax = 0;
        for (auto& kv : st->reqs) {
            const ServeRequest<Real>& r = *kv.second;
            if (r.state != kRunning) continue;
            const size_t n0 = items.size();
            const ProblemClass& pc = r.cd->pc;
            append_items(items, r.first, r.nsolves, pc.nx, pc.ny, pc.nc, item_face_distance(pc), st->blk.T,
                         st->blk.cols, nseg);
            TOMO_TRY(validate_items(items, n0, pc.nx, pc.ny, pc.nc, item_face_distance(pc), st->blk.T, st->blk.cols));
            st->cmax = std::max(st->cmax, dft_contour(pc));
        }
        st->nitems = (int)items.size();
        if (!items.empty()) {
            TOMO_TRY(st->items.ensure(sizeof(WorkItem) * items.size()));
            CUDA_TRY(cudaMemcpyAsync(st->items.p, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice,
                                     stream_));
            TOMO_TRY(advance_grid<Real>(st->blk, advance_mode(cd_.pc.spec), st->nitems, num_sms_, &st->blocks,
                                        &st->smem));
        }
        // the upload vectors must outlive the async copies above
        CUDA_TRY(cudaStreamSynchronize(stream_));
        st->items_dirty = false;
    }
    // 3. advance launches over everything admitted: as many as the running
    // request closest to its end still needs, at most kLaunchesPerStep, so
    // that no request runs past its last step and the host synchronises once
    // per serving step rather than once per launch
    constexpr int kLaunchesPerStep = 4;
    int running = 0;
    if (st->nitems > 0) {
        int nl = kLaunchesPerStep;
        for (auto& kv : st->reqs) {
            const ServeRequest<Real>& r = *kv.second;
            if (r.state == kRunning)
                nl = std::min(nl, (r.cd->pc.S - r.steps_done + st->blk.T - 1) / st->blk.T);
        }
        nl = std::max(nl, 1);
        for (int l = 0; l < nl; ++l)
            launch_advance<Real>(st->blk, advance_mode(cd_.pc.spec), st->blocks, st->smem,
                                 st->descs.template as<SolveDesc<Real>>(), st->items.template as<WorkItem>(),
                                 st->nitems, st->hi_slot, d_counter_.as<int>(), st->cmax, stream_);
        CUDA_TRY(cudaGetLastError());
        for (auto& kv : st->reqs) {
            ServeRequest<Real>& r = *kv.second;
            if (r.state != kRunning) continue;
            r.steps_done += nl * st->blk.T;
            if (r.steps_done >= r.cd->pc.S) TOMO_TRY(retire(st, r, stream_, true));
            else ++running;
        }
    }
    CUDA_TRY(cudaStreamSynchronize(stream_));
    for (auto& kv : st->reqs) {
        ServeRequest<Real>& r = *kv.second;
        if (r.state == kRunning && r.mem == nullptr) {
            r.state = kDone;
            if (r.hflag && r.cd->pc.spec.mode != TOMO_MODE_REFERENCE_GPU) r.status = TOMO_ENUMERIC;
            r.up = Unpacked{};
        }
    }
    int queued = 0, solves = 0;
    for (auto& kv : st->reqs) {
        if (kv.second->state == kQueued) ++queued;
        if (kv.second->state == kRunning) solves += kv.second->nsolves;
    }
    stats_.serve_bytes_in_use = st->bytes_in_use;
    stats_.serve_running = running;
    stats_.serve_queued = queued;
    stats_.serve_running_solves = solves;
    if (n_active) *n_active = running + queued;
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::poll(uint64_t ticket, double* fitness) {
    if (!serve_) return fail(TOMO_EINVAL, "unknown ticket");
    auto it = serve_->reqs.find(ticket);
    if (it == serve_->reqs.end()) return fail(TOMO_EINVAL, "unknown ticket");
    ServeRequest<Real>& r = *it->second;
    if (r.state == kCancelled) {
        serve_->reqs.erase(it);   // reported once, then forgotten
        return fail(TOMO_ECANCELLED, "ticket was cancelled");
    }
    if (r.state == kFailed) {
        const int status = r.status;
        serve_->reqs.erase(it);   // reported once, then forgotten like a finished request
        return fail(status, "request failed");
    }
    if (r.state != kDone) return TOMO_ENOTREADY;
    if (fitness) std::copy(r.fitness.begin(), r.fitness.end(), fitness);
    const int status = r.status;
    serve_->reqs.erase(it);
    if (status) return fail(status, "non-finite field or fitness detected");
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::cancel(uint64_t ticket) {
    if (!serve_) return fail(TOMO_EINVAL, "unknown ticket");
    auto it = serve_->reqs.find(ticket);
    if (it == serve_->reqs.end()) return fail(TOMO_EINVAL, "unknown ticket");
    ServeRequest<Real>& r = *it->second;
    if (r.state == kRunning) {
        TOMO_TRY(retire(serve_, r, stream_, false));
        CUDA_TRY(cudaStreamSynchronize(stream_));
    }
    if (r.state == kQueued || r.state == kRunning) {
        r.state = kCancelled;
        r.up = Unpacked{};   // only the ticket's state is kept until it is polled
    }
    return TOMO_OK;
}

template class EngineT<float>;
template class EngineT<double>;

}  // namespace tomo
