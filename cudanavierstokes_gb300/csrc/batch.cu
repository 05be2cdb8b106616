// batch.cu -- batched ensemble: many simulations of uneven grid sizes advanced together.
// Two execution modes, picked with the launch shape by a measuring autotuner:
//  - persistent: one persistent cooperative launch per Runge-Kutta stage over the work
//    units of all members (and one small launch that advances every member's time at the
//    step start), the step captured in a CUDA graph (one per ping-pong parity);
//  - concurrent: every member advances through its own captured step graph (the
//    standalone stage kernels, coefficients in the launch parameters) on one of up to
//    CNS_BATCH_LANES streams forked from and joined into the batch stream, so the
//    kernels of different members overlap on the device.
//
// Each member is a solver handle (own buffers, scalars and logs); the batch keeps a
// device table of the members' pointers and geometry (BatchInst) and the prefix offsets of
// their work units (BatchCtl). Membership changes rewrite the table in place, so the
// captured graphs stay valid. All members share the stencil orders, the precision and the
// Wray low-storage scheme; each keeps its own dt, CFL/bulk schedule, time and logs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/cns.h"
#include "batch_kernel.cuh"
#include "solver_internal.h"

using namespace cns;

namespace cns {
void launch_batch_stage_fp64(int S, int V, dim3 grid, const BatchInst<double>* tab, const BatchCtl* ctl, int cur,
                             int stage, int quirk, unsigned* bar, int* err, unsigned long long* cnt,
                             const MemberTable<double>& rt, cudaStream_t s);
void launch_batch_stage_fp32(int S, int V, dim3 grid, const BatchInst<float>* tab, const BatchCtl* ctl, int cur,
                             int stage, int quirk, unsigned* bar, int* err, unsigned long long* cnt,
                             const MemberTable<float>& rt, cudaStream_t s);
void launch_batch_time_fp64(const BatchInst<double>* tab, const BatchCtl* ctl, cudaStream_t s);
void launch_batch_time_fp32(const BatchInst<float>* tab, const BatchCtl* ctl, cudaStream_t s);
int batch_stage_occupancy(int fp32, int S, int V, int* blocks_per_sm);
}  // namespace cns

namespace {

const double WA[3] = {0., -17. / 60., -5. / 12.};   // src/cuda_main.cu:10-11
const double WB[3] = {8. / 15., 5. / 12., 3. / 4.};

struct Member {
    cns_solver* h = nullptr;
    int id = -1;
    int64_t steps = 0;      // steps done since admission
    int64_t cap = 0;        // per-step log capacity
};

// execution modes and launch shapes chosen by the autotuner, keyed by precision, stencil
// orders and a size class
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int>> g_tuned;   // -> mode, threads, blocks/SM

int size_class(int64_t points) {
    int c = 0;
    while (points > 1 && c < 40) { points >>= 1; c++; }
    return c;
}

// Exercises the barrier's give-up path: one block waits for a second block that does not
// exist, so the bounded wait must run out and set *err (used by the self test).
__global__ void k_barrier_timeout_probe(unsigned* bar, int* err, long long spin_limit) {
    grid_barrier(bar, 2u, err, spin_limit);
}

}  // namespace

struct cns_batch {
    int device = 0;
    int precision = CNS_PREC_FP64;
    int S = 4, V = 4;
    int quirk = 1;
    int64_t budget = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    std::vector<Member> members;
    int next_id = 0;
    int cur = 0;
    bool dirty = true;
    void* d_tab = nullptr;
    BatchCtl* d_ctl = nullptr;
    unsigned* d_bar = nullptr;
    unsigned long long* d_cnt = nullptr;   // the persistent kernel's four phase unit counters
    std::vector<BatchInst<float>> h_tab32;   // host copy of the FP32 member table (the launch argument's source)
    int* d_err = nullptr;
    int threads = 128, blocks_per_sm = 1, nsm = 152;
    bool tuned = false;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int64_t launches = 0;
    int mode = CNS_BATCH_PERSISTENT;
    std::vector<cudaStream_t> lanes;     // concurrent mode
    std::vector<cudaEvent_t> lane_done;
    cudaEvent_t fork = nullptr;

    void drop_graphs() {
        for (int c = 0; c < 2; c++)
            if (exec[c]) { cudaGraphExecDestroy(exec[c]); exec[c] = nullptr; }
    }
    ~cns_batch() {
        cudaSetDevice(device);
        drop_graphs();
        for (auto& m : members) cns_destroy(m.h);
        if (d_tab) cudaFree(d_tab);
        if (d_ctl) cudaFree(d_ctl);
        if (d_bar) cudaFree(d_bar);
        if (d_cnt) cudaFree(d_cnt);
        if (d_err) cudaFree(d_err);
        for (auto s : lanes) cudaStreamDestroy(s);
        for (auto e : lane_done) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (own_stream) cudaStreamDestroy(own_stream);
    }
};

namespace {

#define BCK(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            char buf_[256];                                                                       \
            snprintf(buf_, sizeof buf_, "%s: %s", #call, cudaGetErrorString(e_));                 \
            return cns::set_error(e_ == cudaErrorMemoryAllocation ? CNS_ERR_OOM : CNS_ERR_CUDA, buf_); \
        }                                                                                         \
    } while (0)

int64_t batch_bytes(const cns_batch* b) {
    int64_t s = 0;
    for (const auto& m : b->members) s += m.h->bytes;
    return s;
}

// device bytes a solver of these parameters will hold (fields x padded volume + tables)
int64_t estimate_bytes(const cns_params& p, int64_t log_steps) {
    const long long G = p.stencil_size, XL = 16;
    const long long P = ((XL + p.mx + G) + 15) / 16 * 16;
    const long long nall = P * (p.my + 2 * G) * (p.mz + 2 * G);
    const bool f32 = p.precision == CNS_PREC_FP32_RHS;
    const long long rs = f32 ? 4 : 8;
    // 2 x 5 FP64 state; derived h, t, p, mu of both state buffers, theta, 5 RK register
    // fields and (FP64) 9 velocity gradients in the RHS type; FP32: 2 x 4 stencil copies
    long long bytes = 10 * nall * 8 + (8 + 1 + 5 + (f32 ? 0 : 9)) * nall * rs + (f32 ? 8 * nall * 4 : 0);
    bytes += (long long)p.mx * p.my * p.mz * 8;   // staging
    bytes += 3 * 8 * (int64_t)std::max<int64_t>(log_steps, 1024) + 64 * 1024;
    return bytes;
}

template <typename R>
BatchInst<R> make_inst(cns_solver* h, int64_t cap) {
    BatchInst<R> I;
    std::memset(&I, 0, sizeof I);
    I.g = h->geom;
    I.ph = h->phys;
    if constexpr (sizeof(R) == 4) I.cf = h->cf32; else I.cf = h->cf64;
    I.scal = h->scal;
    I.tlog = h->tlog;
    for (int c = 0; c < 2; c++) {
        I.in[c] = cns::solver_rhs_in<R>(h, c);
        for (int st = 0; st < 3; st++) I.up[st][c] = cns::solver_stage_update<R>(h, ST_LS, WA[st], WB[st], c);
    }
    I.nbx = (h->p.mx + 31) / 32;
    I.nby = (h->p.my + 3) / 4;
    I.tcap = cap;
    return I;
}

template <typename R>
int upload_table(cns_batch* b) {
    const int n = (int)b->members.size();
    std::vector<BatchInst<R>> tab(std::max(n, 1));
    BatchCtl ctl;
    std::memset(&ctl, 0, sizeof ctl);
    ctl.n = n;
    for (int q = 0; q < n; q++) {
        cns_solver* h = b->members[q].h;
        tab[q] = make_inst<R>(h, b->members[q].cap);
        const long long pu = (long long)tab[q].nbx * tab[q].nby * h->p.mz;
        const long long gc = ghost_count(h->geom);   // the ghost phases' cell count
        ctl.unit_off[q + 1] = ctl.unit_off[q] + pu;
        ctl.ghost_off[q + 1] = ctl.ghost_off[q] + (gc + BATCH_THREADS - 1) / BATCH_THREADS;
    }
    BCK(cudaMemcpyAsync(b->d_tab, tab.data(), sizeof(BatchInst<R>) * n, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_ctl, &ctl, sizeof ctl, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    if constexpr (sizeof(R) == 4) {
        // the member table is a launch argument, baked into the captured steps
        b->h_tab32.assign(tab.begin(), tab.begin() + n);
        b->drop_graphs();
    }
    b->dirty = false;
    return CNS_OK;
}

int upload(cns_batch* b) {
    return b->precision == CNS_PREC_FP32_RHS ? upload_table<float>(b) : upload_table<double>(b);
}

// The persistent kernel's member table for stage s from parity cur: FP32 batches of up to
// MEMBER_TABLE_MAX members (n = 0 otherwise: the kernel reads the device table instead)
MemberTable<float> member_table(const cns_batch* b, int s, int cur) {
    MemberTable<float> t;
    std::memset(&t, 0, sizeof t);
    const int n = (int)b->h_tab32.size();
    if (n > MEMBER_TABLE_MAX) return t;
    t.n = n;
    for (int q = 0; q < n; q++) {
        const BatchInst<float>& I = b->h_tab32[q];
        const RhsIn<float>& in = I.in[cur];
        const Update<float>& up = I.up[s][cur];
        Member32& M = t.m[q];
        M.base = I.g.base; M.P = (int)I.g.P; M.PS = (int)I.g.PS; M.mx = I.g.mx; M.my = I.g.my;
        M.nbx = I.nbx; M.nby = I.nby; M.nonuniform_x = I.g.nonuniform_x;
        M.use_prev = up.use_prev; M.fuse = up.fuse; M.vexp_is_one = up.ph.vexp_is_one;
        for (int d = 0; d < 3; d++) { M.inv[d] = I.cf.inv[d]; M.inv2[d] = I.cf.inv2[d]; }
        M.lam_mu = I.cf.lam_mu; M.ca = up.ca; M.cb = up.cb; M.f_vexp = up.ph.f_vexp; M.f_invRe = up.ph.f_invRe;
        M.cvInv = up.ph.cvInv; M.Rgas = up.ph.Rgas;
        M.xp = I.cf.xp; M.cvsx = I.cf.cvsx;
        M.qa = in.qa; M.qb = in.qb; M.dil = in.dil;
        // the state buffers and the RK register are single blocks with field stride nalloc
        M.fstride = b->members[q].h->nalloc;
        M.qin = up.qin.r; M.qout = up.qout.r; M.rb = up.rb[0];
        M.spx = up.spx; M.spz = up.spz; M.rref = up.rref; M.uref = up.uref; M.vref = up.vref; M.wref = up.wref;
        M.eref = up.eref;
        M.nqa = up.dnext.qa; M.nqb = up.dnext.qb;
        M.scal = I.scal;
        M.G = I.g.G; M.mz = I.g.mz; M.xbc = I.g.xbc; M.zbl = I.g.zbl; M.dy = I.g.dy;
        M.perturbed = I.ph.perturbed; M.pert_kc = I.ph.pert_kc; M.pert_lp = I.ph.pert_lp;
        M.twall_top = I.ph.twall_top; M.twall_bot = I.ph.twall_bot; M.hcoef = I.ph.hcoef; M.invRe = I.ph.invRe;
        M.vexp = I.ph.vexp;
        M.pert_amp1 = I.ph.pert_amp1; M.pert_amp2 = I.ph.pert_amp2; M.pert_omega1 = I.ph.pert_omega1;
        M.pert_omega2 = I.ph.pert_omega2; M.pert_lambda = I.ph.pert_lambda;
        for (int d = 0; d < 3; d++)
            for (int l = 0; l < 5; l++) M.c1V[d][l] = I.cf.c1V[d][l];
        t.unit_off[q + 1] = t.unit_off[q] + (long long)I.nbx * I.nby * I.g.mz;
        t.ghost_off[q + 1] = t.ghost_off[q] + (ghost_count(I.g) + BATCH_THREADS - 1) / BATCH_THREADS;
        t.col_off[q + 1] = t.col_off[q] + (long long)I.nbx * I.nby * ((I.g.mz + COL_NZ - 1) / COL_NZ);
    }
    return t;
}

int launch_stage(cns_batch* b, int s, int cur) {
    const dim3 grid(b->nsm * b->blocks_per_sm);
    const bool f32 = b->precision == CNS_PREC_FP32_RHS;
    if (s == 0) {   // the step's time advance, before the stage reads the time
        if (f32) launch_batch_time_fp32((const BatchInst<float>*)b->d_tab, b->d_ctl, b->stream);
        else launch_batch_time_fp64((const BatchInst<double>*)b->d_tab, b->d_ctl, b->stream);
        b->launches++;
    }
    if (f32)
        launch_batch_stage_fp32(b->S, b->V, grid, (const BatchInst<float>*)b->d_tab, b->d_ctl, cur, s, b->quirk,
                                b->d_bar, b->d_err, b->d_cnt, member_table(b, s, cur), b->stream);
    else
        launch_batch_stage_fp64(b->S, b->V, grid, (const BatchInst<double>*)b->d_tab, b->d_ctl, cur, s, b->quirk,
                                b->d_bar, b->d_err, b->d_cnt, MemberTable<double>{0}, b->stream);
    b->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char buf[200];
        snprintf(buf, sizeof buf, "batch stage launch: %s", cudaGetErrorString(e));
        return cns::set_error(CNS_ERR_CUDA, buf);
    }
    return CNS_OK;
}

// the three stages of one step from parity c, through a captured graph
int step_stages(cns_batch* b) {
    const int c = b->cur;
    if (!b->exec[c]) {
        const int64_t l0 = b->launches;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int rc = CNS_OK;
        for (int s = 0; s < 3 && !rc; s++) rc = launch_stage(b, s, c ^ (s & 1));
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
        b->launches = l0;
        if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
        BCK(e);
        e = cudaGraphInstantiate(&b->exec[c], graph, 0);
        cudaGraphDestroy(graph);
        BCK(e);
    }
    BCK(cudaGraphLaunch(b->exec[c], b->stream));
    b->launches += 4;
    b->cur = c ^ 1;   // three stages: parity flips once per step
    return CNS_OK;
}

// concurrent mode: one step of every member through its own step graph, members spread
// over the lanes (fork from the batch stream, join back into it)
int step_members(cns_batch* b) {
    const int n = (int)b->members.size();
    const int K = std::min(n, CNS_BATCH_LANES);
    while ((int)b->lanes.size() < K) {
        cudaStream_t s = nullptr;
        cudaEvent_t e = nullptr;
        BCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        b->lanes.push_back(s);
        BCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->lane_done.push_back(e);
    }
    if (!b->fork) BCK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    BCK(cudaEventRecord(b->fork, b->stream));
    for (int k = 0; k < K; k++) BCK(cudaStreamWaitEvent(b->lanes[k], b->fork, 0));
    int rc = CNS_OK;
    for (int q = 0; q < n && !rc; q++) {
        cns_solver* h = b->members[q].h;
        h->stream = b->lanes[q % K];
        h->cur = b->cur;
        const int64_t l0 = h->launches;
        rc = cns::solver_step(h);
        b->launches += h->launches - l0;
        h->stream = b->stream;
    }
    for (int k = 0; k < K; k++) {   // join even after an error, so no lane work is left behind
        BCK(cudaEventRecord(b->lane_done[k], b->lanes[k]));
        BCK(cudaStreamWaitEvent(b->stream, b->lane_done[k], 0));
    }
    if (rc) return rc;
    b->cur ^= 1;   // three stages: parity flips once per step
    return CNS_OK;
}

Member* find_member(cns_batch* b, int id) {
    for (auto& m : b->members)
        if (m.id == id) return &m;
    return nullptr;
}

int choose_shape(cns_batch* b) {
    int occ = 0;
    int rc = batch_stage_occupancy(b->precision == CNS_PREC_FP32_RHS, b->S, b->V, &occ);
    if (rc) return rc;
    if (occ < 1) return cns::set_error(CNS_ERR_CUDA, "batch stage kernel cannot be resident");
    if (b->blocks_per_sm > occ) b->blocks_per_sm = occ;
    if (b->blocks_per_sm < 1) b->blocks_per_sm = 1;
    return CNS_OK;
}

}  // namespace

extern "C" {

int cns_batch_create(int device, int precision, int stencil_size, int stencil_visc, int64_t hbm_budget_bytes,
                     cns_batch** out) {
    if (!out) return cns::set_error(CNS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (precision != CNS_PREC_FP64 && precision != CNS_PREC_FP32_RHS)   // the pair mode runs single solvers only
        return cns::set_error(CNS_ERR_INVALID, "batches run in CNS_PREC_FP64 or CNS_PREC_FP32_RHS");
    if (stencil_size < 1 || stencil_size > 4 || stencil_visc < 1 || stencil_visc > stencil_size)
        return cns::set_error(CNS_ERR_INVALID, "stencil orders out of range");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return cns::set_error(CNS_ERR_CUDA, "no CUDA device available");
    }
    if (device < 0 || device >= ndev) return cns::set_error(CNS_ERR_INVALID, "device out of range");
    BCK(cudaSetDevice(device));
    cns_batch* b = new cns_batch();
    b->device = device;
    b->precision = precision;
    b->S = stencil_size;
    b->V = stencil_visc;
    b->budget = hbm_budget_bytes;
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, device);
    cudaError_t e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tab, sizeof(BatchInst<double>) * CNS_BATCH_MAX);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_ctl, sizeof(BatchCtl));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_bar, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_bar, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_cnt, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->d_cnt, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->d_err, 0, sizeof(int));
    if (e != cudaSuccess) {
        delete b;
        return cns::set_error(CNS_ERR_OOM, "batch set-up allocation failed");
    }
    b->stream = b->own_stream;
    int rc = choose_shape(b);
    if (rc) { delete b; return rc; }
    *out = b;
    return CNS_OK;
}

int cns_batch_destroy(cns_batch* b) {
    delete b;
    return CNS_OK;
}

int cns_batch_set_stream(cns_batch* b, void* stream) {
    if (!b) return cns::set_error(CNS_ERR_INVALID, "batch is NULL");
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    for (auto& m : b->members) cns_set_stream(m.h, b->stream);
    return CNS_OK;
}

int cns_batch_add(cns_batch* b, const cns_params* p, const double* r, const double* u, const double* v,
                  const double* w, const double* e, int max_steps, int* id_out) {
    if (!b || !p || !id_out || !r || !u || !v || !w || !e) return cns::set_error(CNS_ERR_INVALID, "NULL argument");
    if ((int)b->members.size() >= CNS_BATCH_MAX) return cns::set_error(CNS_ERR_OOM, "batch is full");
    if (p->stencil_size != b->S || p->stencil_visc != b->V || p->precision != b->precision)
        return cns::set_error(CNS_ERR_INVALID, "member stencil orders / precision differ from the batch");
    if (p->scheme != CNS_RK3_LOWSTORAGE) return cns::set_error(CNS_ERR_INVALID, "batches use the Wray RK3 scheme");
    if (max_steps < 1) return cns::set_error(CNS_ERR_INVALID, "max_steps must be >= 1");
    const int64_t need = estimate_bytes(*p, max_steps);
    if (b->budget > 0 && batch_bytes(b) + need > b->budget)
        return cns::set_error(CNS_ERR_OOM, "HBM budget of the batch would be exceeded");
    BCK(cudaSetDevice(b->device));
    cns_solver* h = nullptr;
    int rc = cns_create(p, b->device, &h);
    if (rc) return rc;
    if (b->budget > 0 && batch_bytes(b) + h->bytes > b->budget) {
        cns_destroy(h);
        return cns::set_error(CNS_ERR_OOM, "HBM budget of the batch would be exceeded");
    }
    cns_set_stream(h, b->stream);
    double* d = nullptr;
    double* t = nullptr;
    const int cap = std::max(max_steps, 16);
    if ((rc = h->alloc(&d, 2 * (size_t)cap)) || (rc = h->alloc(&t, (size_t)cap))) { cns_destroy(h); return rc; }
    h->diag = d; h->tlog = t; h->diag_cap = cap;
    double* arr[5] = {(double*)r, (double*)u, (double*)v, (double*)w, (double*)e};
    rc = cns_copy_field(h, 0, arr[0], arr[1], arr[2], arr[3], arr[4]);
    if (rc) { cns_destroy(h); return rc; }
    solver_set_parity(h, b->cur);
    Member m;
    m.h = h;
    m.id = b->next_id++;
    m.cap = cap;
    b->members.push_back(m);
    b->dirty = true;
    *id_out = m.id;
    return CNS_OK;
}

cns_solver* cns_batch_member(cns_batch* b, int id) {
    Member* m = b ? find_member(b, id) : nullptr;
    if (!m) return nullptr;
    m->h->cur = b->cur;
    b->dirty = true;   // the caller may change the member (e.g. its sponge): rebuild the table
    return m->h;
}

int cns_batch_remove(cns_batch* b, int id) {
    if (!b) return cns::set_error(CNS_ERR_INVALID, "batch is NULL");
    for (size_t q = 0; q < b->members.size(); q++)
        if (b->members[q].id == id) {
            BCK(cudaStreamSynchronize(b->stream));
            cns_destroy(b->members[q].h);
            b->members.erase(b->members.begin() + q);
            b->dirty = true;
            return CNS_OK;
        }
    return cns::set_error(CNS_ERR_INVALID, "no batch member with this id");
}

int cns_batch_get_fields(cns_batch* b, int id, double* r, double* u, double* v, double* w, double* e) {
    cns_solver* h = cns_batch_member(b, id);
    if (!h) return cns::set_error(CNS_ERR_INVALID, "no batch member with this id");
    return cns_copy_field(h, 1, r, u, v, w, e);
}

int cns_batch_get_logs(cns_batch* b, int id, int n, double* par1, double* par2, double* time, double* dt) {
    Member* m = b ? find_member(b, id) : nullptr;
    if (!m) return cns::set_error(CNS_ERR_INVALID, "no batch member with this id");
    BCK(cudaSetDevice(b->device));
    BCK(cudaStreamSynchronize(b->stream));
    const int64_t avail = std::min<int64_t>(m->steps, m->cap);
    if (n > avail) n = (int)avail;
    if (n <= 0) return CNS_OK;
    cns_solver* h = m->h;
    std::vector<double> d(2 * (size_t)n);
    BCK(cudaMemcpy(d.data(), h->diag, d.size() * 8, cudaMemcpyDeviceToHost));
    for (int s = 0; s < n; s++) {
        const bool has = s % h->p.check_bulk == 0;
        if (par1) par1[s] = has ? d[2 * s] : NAN;
        if (par2) par2[s] = has ? d[2 * s + 1] : NAN;
    }
    if (time) BCK(cudaMemcpy(time, h->tlog, (size_t)n * 8, cudaMemcpyDeviceToHost));
    if (dt) {
        double sc[SC_COUNT];
        BCK(cudaMemcpy(sc, h->scal, sizeof sc, cudaMemcpyDeviceToHost));
        *dt = sc[SC_DT];
    }
    return CNS_OK;
}

int cns_batch_info(cns_batch* b, int* count, int64_t* points, int64_t* bytes, int64_t* launches) {
    if (!b) return cns::set_error(CNS_ERR_INVALID, "batch is NULL");
    int64_t pts = 0;
    for (auto& m : b->members) pts += (int64_t)m.h->p.mx * m.h->p.my * m.h->p.mz;
    if (count) *count = (int)b->members.size();
    if (points) *points = pts;
    if (bytes) *bytes = batch_bytes(b);
    if (launches) {
        int64_t l = b->launches;
        for (auto& m : b->members) l += m.h->launches;
        *launches = l;
    }
    return CNS_OK;
}

int cns_batch_member_steps(cns_batch* b, int id, int64_t* steps) {
    Member* m = b ? find_member(b, id) : nullptr;
    if (!m || !steps) return cns::set_error(CNS_ERR_INVALID, "no batch member with this id");
    *steps = m->steps;
    return CNS_OK;
}

int cns_batch_step(cns_batch* b, int nsteps) {
    if (!b) return cns::set_error(CNS_ERR_INVALID, "batch is NULL");
    if (nsteps < 0) return cns::set_error(CNS_ERR_INVALID, "nsteps < 0");
    if (b->members.empty() || nsteps == 0) return CNS_OK;
    BCK(cudaSetDevice(b->device));
    int rc;
    if (b->dirty && (rc = upload(b))) return rc;
    for (int s = 0; s < nsteps; s++) {
        // per-member dt / body force / bulk diagnostics on each member's own schedule
        for (auto& m : b->members) {
            cns_solver* h = m.h;
            h->cur = b->cur;
            // the persistent stages read the current state's derived fields (recovered by
            // the previous stage, or here after a copy-in or an admission)
            if (b->mode == CNS_BATCH_PERSISTENT && (rc = cns::solver_ensure_state(h))) return rc;
            int want = 0;
            double* dg = nullptr;
            const int64_t st = m.steps;
            if (st % h->p.check_cfl == 0) want |= RED_DT | (h->p.forcing ? RED_FORCE : 0);
            if (st % h->p.check_bulk == 0 && st < m.cap) {
                want |= h->p.forcing ? (RED_FORCE | RED_ENERGY) : RED_KE;
                dg = h->diag;
            }
            if (want && (rc = cns::solver_reduce(h, want, dg))) return rc;
        }
        const int c0 = b->cur;
        if ((rc = b->mode == CNS_BATCH_CONCURRENT ? step_members(b) : step_stages(b))) return rc;
        for (auto& m : b->members) {
            m.steps++;
            if (b->mode != CNS_BATCH_CONCURRENT) {
                // as after the standalone fused stages: both derived buffers match their
                // states, and the latest recovery in the reference's order is that of the
                // last stage's input state (buffer c0)
                m.h->der_ok[0] = m.h->der_ok[1] = true;
                m.h->mu_buf = c0;
                m.h->cur = b->cur;
            }
        }
    }
    BCK(cudaStreamSynchronize(b->stream));
    int err = 0;
    BCK(cudaMemcpy(&err, b->d_err, sizeof err, cudaMemcpyDeviceToHost));
    if (err) {
        cudaMemset(b->d_err, 0, sizeof(int));
        cudaMemset(b->d_bar, 0, 2 * sizeof(unsigned));
        cudaMemset(b->d_cnt, 0, 4 * sizeof(unsigned long long));
        return cns::set_error(CNS_ERR_TIMEOUT, "batch grid barrier gave up (bounded wait)");
    }
    for (auto& m : b->members) {
        double sc[SC_COUNT];
        BCK(cudaMemcpy(sc, m.h->scal, sizeof sc, cudaMemcpyDeviceToHost));
        if (sc[SC_NONFINITE] != 0.0) {
            char buf[160];
            snprintf(buf, sizeof buf, "batch member %d: non-positive or non-finite density/temperature", m.id);
            return cns::set_error(CNS_ERR_NONFINITE, buf);
        }
    }
    return CNS_OK;
}

int cns_batch_set_shape(cns_batch* b, int threads, int blocks_per_sm) {
    if (!b || threads != BATCH_THREADS || blocks_per_sm < 1)
        return cns::set_error(CNS_ERR_INVALID, "threads must be 128, blocks_per_sm >= 1");
    b->threads = threads;
    b->blocks_per_sm = blocks_per_sm;
    int rc = choose_shape(b);
    if (rc) return rc;
    b->drop_graphs();
    b->dirty = true;
    return CNS_OK;
}

int cns_batch_set_mode(cns_batch* b, int mode) {
    if (!b || (mode != CNS_BATCH_PERSISTENT && mode != CNS_BATCH_CONCURRENT))
        return cns::set_error(CNS_ERR_INVALID, "mode must be CNS_BATCH_PERSISTENT or CNS_BATCH_CONCURRENT");
    b->mode = mode;
    return CNS_OK;
}

int cns_batch_get_mode(cns_batch* b, int* mode) {
    if (!b || !mode) return cns::set_error(CNS_ERR_INVALID, "NULL argument");
    *mode = b->mode;
    return CNS_OK;
}

int cns_batch_get_shape(cns_batch* b, int* threads, int* blocks_per_sm) {
    if (!b) return cns::set_error(CNS_ERR_INVALID, "batch is NULL");
    if (threads) *threads = b->threads;
    if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
    return CNS_OK;
}

// Measure each execution mode and launch shape on the current members (advancing them by
// `steps` steps per candidate) and keep the fastest; results are cached per precision,
// stencil orders and size class for later batches.
int cns_batch_tune(cns_batch* b, int steps, double* best_ms) {
    if (!b || steps < 1) return cns::set_error(CNS_ERR_INVALID, "bad arguments");
    if (b->members.empty()) return cns::set_error(CNS_ERR_STATE, "tune needs members");
    int64_t pts = 0;
    for (auto& m : b->members) pts += (int64_t)m.h->p.mx * m.h->p.my * m.h->p.mz;
    const auto key = std::make_tuple(b->precision, b->S, b->V, size_class(pts));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            if (best_ms) *best_ms = -1.0;
            int rc = cns_batch_set_mode(b, std::get<0>(it->second));
            return rc ? rc : cns_batch_set_shape(b, std::get<1>(it->second), std::get<2>(it->second));
        }
    }
    BCK(cudaSetDevice(b->device));
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    double best = 1e30;
    int bm = b->mode, bt = b->threads, bb = b->blocks_per_sm;
    auto measure = [&](int mode, int threads, int bps) -> int {
        int rc = cns_batch_set_mode(b, mode);
        if (!rc && mode == CNS_BATCH_PERSISTENT) rc = cns_batch_set_shape(b, threads, bps);
        if (rc) return CNS_OK;   // shape not available: skip the candidate
        if ((rc = cns_batch_step(b, 1))) return rc;   // capture + warm-up
        BCK(cudaEventRecord(e0, b->stream));
        if ((rc = cns_batch_step(b, steps))) return rc;
        BCK(cudaEventRecord(e1, b->stream));
        BCK(cudaEventSynchronize(e1));
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) { best = ms; bm = mode; bt = b->threads; bb = b->blocks_per_sm; }
        return CNS_OK;
    };
    int rc = measure(CNS_BATCH_CONCURRENT, b->threads, b->blocks_per_sm);
    int occ = 0;
    if (!rc && !batch_stage_occupancy(b->precision == CNS_PREC_FP32_RHS, b->S, b->V, &occ) && occ >= 1) {
        // full residency first, then fewer blocks (less barrier traffic, more cache per block)
        int prev = 0;
        for (int bps : {occ, occ - 2, occ / 2, 1}) {
            if (bps < 1 || bps == prev || rc) continue;
            rc = measure(CNS_BATCH_PERSISTENT, BATCH_THREADS, bps);
            prev = bps;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[key] = std::make_tuple(bm, bt, bb);
    }
    if (best_ms) *best_ms = best / steps;
    rc = cns_batch_set_mode(b, bm);
    return rc ? rc : cns_batch_set_shape(b, bt, bb);
}

// Failure-detection self test of the bounded grid barrier: a one-block launch waits for a
// block that never arrives; the wait must give up after `spin_limit` polls and report it.
int cns_selftest_barrier_timeout(int device, long long spin_limit, int* timed_out) {
    if (!timed_out || spin_limit < 1 || spin_limit > (1LL << 20))
        return cns::set_error(CNS_ERR_INVALID, "spin_limit must be 1..2^20");
    BCK(cudaSetDevice(device));
    unsigned* bar = nullptr;
    int* err = nullptr;
    BCK(cudaMalloc(&bar, 2 * sizeof(unsigned)));
    BCK(cudaMalloc(&err, sizeof(int)));
    cudaMemset(bar, 0, 2 * sizeof(unsigned));
    cudaMemset(err, 0, sizeof(int));
    k_barrier_timeout_probe<<<1, 32>>>(bar, err, spin_limit);
    cudaError_t e = cudaDeviceSynchronize();
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(bar);
    cudaFree(err);
    BCK(e);
    *timed_out = h;
    return CNS_OK;
}

}  // extern "C"
