// Served mode: continuous batching of independent MD jobs on one GPU.
//
// The reference runs one simulation per process (src/fmd.h: one fmd_t per
// run, its time loop in src/integrators.c:227-264).  A request loop here
// keeps many of them resident in HBM at once:
//
//  * a job is a host description (box, kinds, pair table, atoms, steps,
//    dt, precision); it waits in a FIFO queue until the device bytes it
//    needs fit the HBM budget (and a job slot is free);
//  * on admission it becomes an ordinary device system (fmdg_sys_t,
//    stream-ordered allocations on its own stream), its initial forces and
//    thermo record are computed on that stream;
//  * admitted systems of one pair category and precision form a pack; one
//    launch per kernel advances every member by one velocity-Verlet step
//    (LocPack: the systems' geometry in kernel parameters), one step is
//    captured once as a CUDA graph, a chunk replays it `chunk_steps` times,
//    until the membership changes;
//  * every member carries its own step budget on the device (steps_left):
//    a member that has finished is skipped by every kernel, so a chunk
//    needs no host decision in the middle;
//  * up to two chunks per pack are in flight; jobs arriving meanwhile are
//    admitted on their own streams, and a retired job's memory is released
//    stream-ordered, so admission and retirement never stall the device;
//  * the threads per block of the list/density/force kernels are chosen by
//    a small autotuner: the first chunks of each pack try 64, 128 and 256
//    threads and keep the one with the lowest device time per atom-step.
//
// Each member's arithmetic is the single-system arithmetic (one thread per
// atom, fixed list order), so an atom's trajectory does not depend on the
// other members of its pack nor on the tuned block size; only the block
// partial sums of the thermo record are grouped differently.
#include "fmdg_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <vector>

namespace {

enum { JOB_QUEUED = 0, JOB_RUNNING = 1, JOB_DONE = 2, JOB_FAILED = 3 };

struct Job
{
    long long id;
    // description (host copies)
    double l[3];
    int pbc[3];
    int nkinds;
    double mass[FMDG_MAXK];
    int elem[FMDG_MAXK];
    fmdg_pair_t pairs[FMDG_MAXK * FMDG_MAXK];
    int eam_key;
    int n;
    std::vector<double> x, v;
    std::vector<unsigned> kind;
    int steps;
    double dt;
    int prec;
    int keep_state;
    int cats;           // bit mask (1 << FMDG_POT_*) of the pair categories
    double skin;        // Verlet skin of the job's list (fixed at submission)
    int list_capacity;  // list entries per atom, 0: estimated (fixed at submission)
    int nc[3];
    double cellh[3];
    double rcmax;
    std::vector<int> order, cell_count;   // host binning (upload order)
    // runtime
    fmdg_sys_t *sys = nullptr;
    size_t bytes = 0;
    int left = 0;       // steps not yet enqueued
    int refs = 0;       // in-flight chunks that contain it
    int state = JOB_QUEUED;
    int fail_code = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    fmdg_thermo_t th0, th1;
    fmdg_thermo_t *th0_pin = nullptr;   // pinned landing place of th0 until retirement
    unsigned errs = 0;
    cudaEvent_t ready = nullptr;
    std::vector<double> fx, fv, fF;
    std::vector<unsigned> fid;
};

struct Chunk
{
    long long seq;
    cudaEvent_t ev0, ev1;
    std::vector<Job *> members;
    double atom_steps;
    int fblk;
    bool timed;         // counts for the tuner
};

// At most FMDG_PACK_MAX systems (their Geo travel as kernel parameters);
// more systems of one class and precision form further packs, each on its
// own stream.  Class: the pair category of single-category jobs
// (FMDG_POT_LJ, _EAM, _MORSE), 0 for jobs that mix categories (hybrid).
struct Pack
{
    int cls = 0, mixed = 0;
    int lean = 0;       // one-kind jobs (lean binary32 kernels); a job's variant never depends on the mix
    cudaStream_t stream = nullptr;
    std::vector<Job *> members;
    bool dirty = true;
    fmdg_pack_launch P;
    cudaGraphExec_t exec = nullptr;
    int exec_fblk = 0;
    int exec_kernels = 0;          // kernels per replay of the chunk graph
    std::deque<Chunk> inflight;
    std::vector<std::pair<long long, cudaGraphExec_t>> old_execs;   // (last chunk seq, exec)
    long long chunks = 0, rebuilds = 0;
    double atom_steps = 0.0;
    int active() const
    {
        int a = 0;
        for (const Job *j : members) a += j->left > 0;
        return a;
    }
};

// block-size autotuner of one class and precision (shared by its packs)
struct Tuner
{
    int fblk = 128;
    bool tuned = false;
    int step = 0;
    double cost[3] = {1e300, 1e300, 1e300};
};

const int TUNE_BLK[3] = {64, 128, 256};
const int TUNE_ROUNDS = 6;   // chunks measured before the choice (2 per candidate)

double wall_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

} // namespace

struct fmdg_server
{
    int device;
    size_t budget, used = 0, peak = 0;
    int max_jobs, chunk;
    int fixed_fblk = 0;               // 0: autotune
    double skin = 0.8;                // Verlet skin of the packed neighbour lists (A)
    int list_capacity = 0;            // list entries per atom, 0: estimated per job
    double t0;
    long long next_id = 1, seq = 0;
    std::deque<Job *> queue;
    std::map<long long, Job *> jobs;
    int running = 0;
    std::vector<Pack *> packs[4][2];  // [class][mixed]
    Tuner tuners[4][2];
    std::map<int, fmdg_sys_t *> eam_owner;   // shared EAM tables by key
    std::vector<cudaEvent_t> free_events;
    std::vector<fmdg_thermo_t *> free_pins;   // pinned host thermo records (admission)
    std::vector<void *> pin_blocks;
    long long admitted = 0, finished = 0, failed = 0;
    long long kernels = 0;            // kernels launched (graph replays included)
    double atom_steps_done = 0.0;
    cudaStream_t join = nullptr;      // timing of the resident-fleet steps
    cudaEvent_t jev0 = nullptr, jev1 = nullptr;
};

namespace {

cudaEvent_t get_event(fmdg_server_t *S)
{
    if (!S->free_events.empty())
    {
        cudaEvent_t e = S->free_events.back();
        S->free_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void put_event(fmdg_server_t *S, cudaEvent_t e) { if (e) S->free_events.push_back(e); }

// pinned host records, allocated 256 at a time (cudaMallocHost is slow)
fmdg_thermo_t *get_pin(fmdg_server_t *S)
{
    if (S->free_pins.empty())
    {
        void *b = nullptr;
        if (cudaMallocHost(&b, 256 * sizeof(fmdg_thermo_t)) != cudaSuccess) return nullptr;
        S->pin_blocks.push_back(b);
        for (int k = 255; k >= 0; k--) S->free_pins.push_back((fmdg_thermo_t *)b + k);
    }
    fmdg_thermo_t *p = S->free_pins.back();
    S->free_pins.pop_back();
    return p;
}

// the job's initial thermo record, once its stream has drained
void take_th0(fmdg_server_t *S, Job *j)
{
    if (!j->th0_pin) return;
    j->th0 = *j->th0_pin;
    S->free_pins.push_back(j->th0_pin);
    j->th0_pin = nullptr;
}

template <typename F>
void each_pack(fmdg_server_t *S, F f)
{
    for (auto &row : S->packs)
        for (auto &v : row)
            for (Pack *p : v) f(*p);
}

int want_fblk(const fmdg_server_t *S, const Pack &p)
{
    if (S->fixed_fblk) return S->fixed_fblk;
    const Tuner &t = S->tuners[p.cls][p.mixed];
    return t.tuned ? t.fblk : TUNE_BLK[t.step % 3];
}

int pack_class(int cats) { return __builtin_popcount(cats) > 1 ? 0 : __builtin_ctz(cats); }

// a pack of (class, mixed, lean) with room for one more system
Pack *pack_for(fmdg_server_t *S, int cls, int mixed, int lean)
{
    for (Pack *p : S->packs[cls][mixed])
        if (p->lean == lean && p->active() < FMDG_PACK_MAX) return p;
    Pack *p = new Pack();
    p->cls = cls;
    p->mixed = mixed;
    p->lean = lean;
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        delete p;
        return nullptr;
    }
    S->packs[cls][mixed].push_back(p);
    return p;
}

// admitted: the job's bytes and slot were counted
int fail_job(fmdg_server_t *S, Job *j, int code, bool admitted)
{
    j->state = JOB_FAILED;
    j->fail_code = code;
    j->t_done = wall_s() - S->t0;
    if (j->sys)
    {
        fmdg_destroy(j->sys);   // (drains the job's stream)
        j->sys = nullptr;
    }
    take_th0(S, j);
    if (j->ready)
    {
        put_event(S, j->ready);
        j->ready = nullptr;
    }
    if (admitted)
    {
        S->used -= j->bytes;
        S->running--;
    }
    S->failed++;
    return code;
}

// Create the device system of a job (src/misc.c:41-62 cell grid; the atoms
// binned on the host in input order inside each cell).
int setup_job(fmdg_server_t *S, Job *j)
{
    int rc = fmdg_create(&j->sys, S->device);
    if (rc) return rc;
    fmdg_sys_t *s = j->sys;
    if ((rc = fmdg_set_box(s, j->l, j->pbc, j->nc, j->cellh))) return rc;
    if ((rc = fmdg_set_skin(s, j->skin))) return rc;
    if ((rc = fmdg_set_list_capacity(s, j->list_capacity))) return rc;
    if ((rc = fmdg_set_kinds(s, j->nkinds, j->mass, j->elem))) return rc;
    if ((rc = fmdg_set_pairs(s, j->pairs))) return rc;
    if (j->cats & (1 << FMDG_POT_EAM))
    {
        auto it = S->eam_owner.find(j->eam_key);
        if (it == S->eam_owner.end()) return fmdg_set_error("fmdg_srv: unknown EAM table key");
        if ((rc = fmdg_share_eam(s, it->second))) return rc;
    }
    if ((rc = fmdg_set_precision(s, j->prec))) return rc;
    std::vector<double> hx(3 * (size_t)j->n), hv(3 * (size_t)j->n);
    std::vector<unsigned> hk(j->n), hid(j->n);
    std::vector<int> hg(j->n, 0);
    for (int k = 0; k < j->n; k++)
    {
        const int a = j->order[k];
        for (int d = 0; d < 3; d++)
        {
            hx[3 * (size_t)k + d] = j->x[3 * (size_t)a + d];
            hv[3 * (size_t)k + d] = j->v[3 * (size_t)a + d];
        }
        hk[k] = j->kind[a];
        hid[k] = (unsigned)a;
    }
    if ((rc = fmdg_upload(s, j->n, j->cell_count.data(), hx.data(), hv.data(), hk.data(), hg.data(), hid.data())))
        return rc;
    // the packed kernels walk skin lists only
    if (!s->g.skin_on) return fmdg_set_error("fmdg_srv: the job's box admits no skin list");
    if ((rc = fmdg_compute_forces(s, -1))) return rc;
    // the initial thermo record lands in pinned host memory on the job's
    // stream and is read at retirement: admission never waits for the GPU,
    // which is busy with the packed chunks
    if ((rc = fmdg_launch_thermo(s, -1, 0, 0.0, 1.0, 0.0))) return rc;
    if (!(j->th0_pin = get_pin(S))) return fmdg_set_error("fmdg_srv: cannot allocate pinned host memory");
    FMDG_CK(cudaMemcpyAsync(j->th0_pin, s->g.thermo, sizeof(fmdg_thermo_t), cudaMemcpyDeviceToHost, s->stream));
    if ((rc = fmdg_set_steps_left(s, j->steps))) return rc;
    set_step_dt(s, j->dt);
    s->g.st.tau = 1.0;
    s->g.st.T0 = 0.0;
    s->g.st.group = -1;
    s->g.st.thermostat = 0;
    j->ready = get_event(S);
    FMDG_CK(cudaEventRecord(j->ready, s->stream));
    return FMDG_OK;
}

int retire(fmdg_server_t *S, Job *j);

// Admits queued jobs in FIFO order while they fit; at most `budget_s` of
// host time per call (0: no limit), so a serving loop keeps launching
// chunks between admissions.
int admit(fmdg_server_t *S, double budget_s)
{
    const double t_end = wall_s() + budget_s;
    while (!S->queue.empty() && (budget_s <= 0.0 || wall_s() < t_end))
    {
        Job *j = S->queue.front();
        if (j->bytes > S->budget)
        {
            S->queue.pop_front();
            fail_job(S, j, FMDG_E_NOMEM, false);
            continue;
        }
        if (S->running >= S->max_jobs || S->used + j->bytes > S->budget) break;
        S->queue.pop_front();
        S->used += j->bytes;
        S->peak = std::max(S->peak, S->used);
        S->running++;
        const int rc = setup_job(S, j);
        if (rc)
        {
            fail_job(S, j, rc, true);
            continue;
        }
        j->state = JOB_RUNNING;
        j->t_start = wall_s() - S->t0;
        j->left = j->steps;
        S->admitted++;
        if (j->left == 0)
        {
            retire(S, j);
            continue;
        }
        Pack *p = pack_for(S, pack_class(j->cats), j->prec == FMDG_PREC_MIXED, j->nkinds == 1);
        if (!p)
        {
            fail_job(S, j, fmdg_set_error("fmdg_srv: cannot create a pack stream"), true);
            continue;
        }
        p->members.push_back(j);
        p->dirty = true;
    }
    return FMDG_OK;
}

// Geo table, block maps and the captured chunk of the current membership.
int rebuild(fmdg_server_t *S, Pack &p)
{
    std::vector<Job *> keep;
    for (Job *j : p.members)
        if (j->left > 0) keep.push_back(j);
    p.members.swap(keep);
    p.dirty = false;
    if (p.exec)
    {
        p.old_execs.push_back({S->seq, p.exec});   // freed once chunk S->seq-1 and older are done
        p.exec = nullptr;
    }
    if (p.members.empty()) return FMDG_OK;
    const int fblk = want_fblk(S, p);
    fmdg_pack_launch &P = p.P;
    P.stream = p.stream;
    P.nsys = (int)p.members.size();
    P.cats = 0;
    for (const Job *j : p.members) P.cats |= j->cats;
    P.lean = p.lean;
    P.mixed = p.mixed;
    P.fblk = fblk;
    LocPack *locs[4] = {&P.la, &P.lc, &P.lf, &P.ls};
    for (LocPack *L : locs)
    {
        L->nsys = P.nsys;
        L->bstart[0] = 0;
    }
    for (int k = 0; k < P.nsys; k++)
    {
        fmdg_sys_t *s = p.members[k]->sys;
        s->fblk = fblk;
        for (LocPack *L : locs) L->geos[k] = s->g;
        P.la.bstart[k + 1] = P.la.bstart[k] + fmdg_grid(s->g.cap, 128);
        P.lc.bstart[k + 1] = P.lc.bstart[k] + fmdg_grid(s->g.ncell, 128);
        P.lf.bstart[k + 1] = P.lf.bstart[k] + fmdg_grid(s->g.cap, fblk);
        P.ls.bstart[k + 1] = k + 1;
    }
    // members set up on their own streams must be ready before the chunk
    for (Job *j : p.members)
        if (j->ready) FMDG_CK(cudaStreamWaitEvent(p.stream, j->ready, 0));
    cudaGraph_t graph;
    FMDG_CK(cudaStreamBeginCapture(p.stream, cudaStreamCaptureModeThreadLocal));
    // one step per graph, replayed chunk_steps times: a membership change
    // re-captures 10-11 kernels, not chunk_steps times as many
    int rc = FMDG_OK, nk = 0;
    {
        int a = fmdg_pack_launch_refresh(P);
        int b = a < 0 ? a : fmdg_pack_launch_forces(P, 7);
        if (a < 0 || b < 0) rc = -(a < 0 ? a : b);
        else nk = a + b;
    }
    cudaError_t e = cudaStreamEndCapture(p.stream, &graph);
    if (rc) return rc;
    p.exec_kernels = nk;
    if (e != cudaSuccess) return fmdg_fail("cudaStreamEndCapture", e);
    e = cudaGraphInstantiate(&p.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fmdg_fail("cudaGraphInstantiate", e);
    p.exec_fblk = fblk;
    p.rebuilds++;
    return FMDG_OK;
}

int launch_chunk(fmdg_server_t *S, Pack &p)
{
    if (p.exec && p.exec_fblk != want_fblk(S, p)) p.dirty = true;
    if (p.dirty)
    {
        int rc = rebuild(S, p);
        if (rc) return rc;
    }
    if (p.members.empty() || !p.exec) return FMDG_OK;
    Chunk c;
    c.seq = S->seq++;
    c.ev0 = get_event(S);
    c.ev1 = get_event(S);
    c.fblk = p.exec_fblk;
    c.atom_steps = 0.0;
    c.members = p.members;
    FMDG_CK(cudaEventRecord(c.ev0, p.stream));
    for (int k = 0; k < S->chunk; k++) FMDG_CK(cudaGraphLaunch(p.exec, p.stream));
    FMDG_CK(cudaEventRecord(c.ev1, p.stream));
    S->kernels += (long long)p.exec_kernels * S->chunk;
    bool full = true;
    for (Job *j : c.members)
    {
        const int k = std::min(S->chunk, j->left);
        if (k < S->chunk) full = false;
        j->left -= k;
        j->refs++;
        c.atom_steps += (double)j->n * k;
        if (j->left == 0) p.dirty = true;
    }
    c.timed = full && !S->tuners[p.cls][p.mixed].tuned && !S->fixed_fblk;
    p.inflight.push_back(c);
    p.chunks++;
    return FMDG_OK;
}

int retire(fmdg_server_t *S, Job *j)
{
    fmdg_sys_t *s = j->sys;
    int rc = fmdg_get_thermo(s, &j->th1);   // (drains the job's stream)
    take_th0(S, j);
    if (!rc) rc = fmdg_get_errors(s, &j->errs, 0);
    if (!rc && j->keep_state)
    {
        int n = 0;
        fmdg_natoms(s, &n);
        j->fx.resize(3 * (size_t)n);
        j->fv.resize(3 * (size_t)n);
        j->fF.resize(3 * (size_t)n);
        j->fid.resize(n);
        rc = fmdg_download(s, nullptr, j->fx.data(), j->fv.data(), j->fF.data(), nullptr, nullptr, nullptr,
                           j->fid.data());
        // packed systems refresh their cells on list rebuilds only: an atom
        // that crossed a periodic face since then is brought back into the
        // box as a refresh would (x -/+ l)
        for (int a = 0; a < n && !rc; a++)
            for (int d = 0; d < 3; d++)
            {
                double &x = j->fx[3 * (size_t)a + d];
                if (!j->pbc[d]) continue;
                if (x >= j->l[d]) x = x - j->l[d];
                else if (x < 0.0) x = x + j->l[d];
            }
    }
    put_event(S, j->ready);
    j->ready = nullptr;
    fmdg_destroy(s);
    j->sys = nullptr;
    S->used -= j->bytes;
    S->running--;
    j->t_done = wall_s() - S->t0;
    if (rc)
    {
        j->state = JOB_FAILED;
        j->fail_code = rc;
        S->failed++;
        return rc;
    }
    j->state = JOB_DONE;
    S->finished++;
    return FMDG_OK;
}

// Completed chunks: tuner samples, finished jobs, graphs no longer used.
int reap(fmdg_server_t *S, Pack &p, bool block)
{
    while (!p.inflight.empty())
    {
        Chunk &c = p.inflight.front();
        if (block)
        {
            FMDG_CK(cudaEventSynchronize(c.ev1));
            block = false;
        }
        const cudaError_t q = cudaEventQuery(c.ev1);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) return fmdg_fail("chunk", q);
        Tuner &t = S->tuners[p.cls][p.mixed];
        if (c.timed && !t.tuned && c.atom_steps > 0)
        {
            // device time per atom-step of this block size; the next chunks
            // of the category try the next candidate (or keep the choice)
            float ms = 0.f;
            cudaEventElapsedTime(&ms, c.ev0, c.ev1);
            const int slot = (c.fblk == 64) ? 0 : (c.fblk == 128 ? 1 : 2);
            t.cost[slot] = std::min(t.cost[slot], ms / c.atom_steps);
            t.step++;
            if (t.step >= TUNE_ROUNDS)
            {
                int best = 1;
                for (int k = 0; k < 3; k++)
                    if (t.cost[k] < t.cost[best]) best = k;
                t.fblk = TUNE_BLK[best];
                t.tuned = true;
            }
        }
        p.atom_steps += c.atom_steps;
        S->atom_steps_done += c.atom_steps;
        for (Job *j : c.members)
        {
            j->refs--;
            if (j->left == 0 && j->refs == 0 && j->state == JOB_RUNNING)
            {
                int rc = retire(S, j);
                (void)rc;
            }
        }
        const long long done_seq = c.seq;
        put_event(S, c.ev0);
        put_event(S, c.ev1);
        p.inflight.pop_front();
        for (size_t k = 0; k < p.old_execs.size();)
        {
            if (p.old_execs[k].first <= done_seq + 1)
            {
                cudaGraphExecDestroy(p.old_execs[k].second);
                p.old_execs.erase(p.old_execs.begin() + k);
            }
            else
                k++;
        }
    }
    return FMDG_OK;
}

} // namespace

extern "C" int fmdg_srv_create(fmdg_server_t **out, int device, size_t hbm_budget, int max_jobs, int chunk_steps)
{
    *out = nullptr;
    if (chunk_steps < 1 || max_jobs < 1) return fmdg_set_error("fmdg_srv_create: bad limits");
    FMDG_CK(cudaSetDevice(device));
    fmdg_server_t *S = new fmdg_server_t();
    S->device = device;
    S->budget = hbm_budget;
    S->max_jobs = max_jobs;
    S->chunk = chunk_steps;
    S->t0 = wall_s();
    *out = S;
    return FMDG_OK;
}

extern "C" void fmdg_srv_destroy(fmdg_server_t *S)
{
    if (!S) return;
    cudaSetDevice(S->device);
    each_pack(S, [&](Pack &p) {
        cudaStreamSynchronize(p.stream);
        for (Chunk &c : p.inflight) { cudaEventDestroy(c.ev0); cudaEventDestroy(c.ev1); }
        if (p.exec) cudaGraphExecDestroy(p.exec);
        for (auto &oe : p.old_execs) cudaGraphExecDestroy(oe.second);
        cudaStreamDestroy(p.stream);
    });
    for (auto &row : S->packs)
        for (auto &v : row)
            for (Pack *p : v) delete p;
    for (auto &kv : S->jobs)
    {
        Job *j = kv.second;
        if (j->sys) fmdg_destroy(j->sys);
        if (j->ready) cudaEventDestroy(j->ready);
        delete j;
    }
    for (auto &kv : S->eam_owner) fmdg_destroy(kv.second);
    for (cudaEvent_t e : S->free_events) cudaEventDestroy(e);
    for (void *b : S->pin_blocks) cudaFreeHost(b);
    if (S->join) cudaStreamDestroy(S->join);
    if (S->jev0) cudaEventDestroy(S->jev0);
    if (S->jev1) cudaEventDestroy(S->jev1);
    delete S;
}

extern "C" int fmdg_srv_set_eam(fmdg_server_t *S, int key, int nelem, int Nrho, double drho, int Nr2, double dr2,
                                const double *F, const double *F_DD, const double *rho, const double *rhoDD,
                                const double *phi, const double *phiDD)
{
    if (S->eam_owner.count(key)) return fmdg_set_error("fmdg_srv_set_eam: key in use");
    fmdg_sys_t *o = nullptr;
    int rc = fmdg_create(&o, S->device);
    if (rc) return rc;
    if ((rc = fmdg_set_eam(o, nelem, Nrho, drho, Nr2, dr2, F, F_DD, rho, rhoDD, phi, phiDD)))
    {
        fmdg_destroy(o);
        return rc;
    }
    S->eam_owner[key] = o;
    return FMDG_OK;
}

extern "C" int fmdg_srv_set_tuning(fmdg_server_t *S, int fblk)
{
    if (fblk != 0 && fblk != 64 && fblk != 128 && fblk != 256)
        return fmdg_set_error("fmdg_srv_set_tuning: 0 (autotune), 64, 128 or 256");
    S->fixed_fblk = fblk;
    each_pack(S, [](Pack &p) { p.dirty = true; });
    return FMDG_OK;
}

extern "C" int fmdg_srv_set_skin(fmdg_server_t *S, double skin)
{
    if (!(skin > 0.0 && skin < 5.0)) return fmdg_set_error("fmdg_srv_set_skin: skin in (0, 5) A");
    S->skin = skin;
    return FMDG_OK;
}

extern "C" int fmdg_srv_set_list_capacity(fmdg_server_t *S, int entries)
{
    if (entries < 0 || entries > 1024 || (entries % 8) != 0)
        return fmdg_set_error("fmdg_srv_set_list_capacity: 0 or a multiple of 8 up to 1024");
    S->list_capacity = entries;
    return FMDG_OK;
}

extern "C" int fmdg_srv_submit(fmdg_server_t *S, const fmdg_job_desc_t *d, long long *id)
{
    if (d->nkinds < 1 || d->nkinds > FMDG_MAXK) return fmdg_set_error("fmdg_srv_submit: 1..8 kinds");
    if (d->n < 1 || d->steps < 0 || !(d->dt > 0.0)) return fmdg_set_error("fmdg_srv_submit: bad n, steps or dt");
    if (d->precision != FMDG_PREC_FP64 && d->precision != FMDG_PREC_MIXED)
        return fmdg_set_error("fmdg_srv_submit: bad precision");
    Job *j = new Job();
    const int nk2 = d->nkinds * d->nkinds;
    int cats = 0;
    double rc2max = 0.0;
    for (int k = 0; k < nk2; k++)
    {
        const fmdg_pair_t &pp = d->pairs[k];
        if (pp.cat != FMDG_POT_LJ && pp.cat != FMDG_POT_MORSE && pp.cat != FMDG_POT_EAM)
        {
            delete j;
            return fmdg_set_error("fmdg_srv_submit: every kind pair needs a potential");
        }
        cats |= 1 << pp.cat;
        rc2max = std::max(rc2max, pp.cat == FMDG_POT_MORSE ? pp.p[3] : pp.p[2]);
        j->pairs[k] = pp;
    }
    j->cats = cats;
    if (cats & (1 << FMDG_POT_EAM))
    {
        // EAM pairs read the shared tables of eam_key: both kinds need an
        // element of those tables, and so do the pair's table indices
        auto it = S->eam_owner.find(d->eam_key);
        if (it == S->eam_owner.end())
        {
            delete j;
            return fmdg_set_error("fmdg_srv_submit: EAM job with an unknown table key");
        }
        const int ne = it->second->g.nelem;
        for (int a = 0; a < d->nkinds; a++)
            for (int b = 0; b < d->nkinds; b++)
            {
                const fmdg_pair_t &pp = d->pairs[a * d->nkinds + b];
                if (pp.cat != FMDG_POT_EAM) continue;
                const int ea = d->eam_elem ? d->eam_elem[a] : -1, eb = d->eam_elem ? d->eam_elem[b] : -1;
                if (ea < 0 || ea >= ne || eb < 0 || eb >= ne || pp.iloc < 0 || pp.iloc >= ne || pp.jloc < 0 ||
                    pp.jloc >= ne)
                {
                    delete j;
                    return fmdg_set_error("fmdg_srv_submit: an EAM pair without elements of the tables");
                }
            }
    }
    const double rcmax = sqrt(rc2max);
    j->rcmax = rcmax;
    for (int k = 0; k < 3; k++)
        if (d->pbc[k] && !(d->l[k] > 2.0 * rcmax))
        {
            delete j;
            return fmdg_set_error("fmdg_srv_submit: a periodic box length is not above twice the cutoff");
        }
    // The job's skin (fixed now): at most 0.99 rc, the list radius rc + skin
    // below half of every periodic box length.
    double skin = std::min(S->skin, 0.99 * rcmax);
    for (int k = 0; k < 3; k++)
        if (d->pbc[k]) skin = std::min(skin, 0.9 * (0.5 * d->l[k] - rcmax));
    j->skin = skin;
    j->list_capacity = S->list_capacity;
    const double rl = rcmax + skin;
    // Cell grid of the reference (src/misc.c:41-50): nc = (int)(l/rc_max),
    // cellh = l/nc.  (Cells of half the list radius were measured too: list
    // builds 20-30% faster, pair forces slower -- their gathers spread over
    // more, smaller cells -- no net gain.)
    for (int k = 0; k < 3; k++)
    {
        j->l[k] = d->l[k];
        j->pbc[k] = d->pbc[k];
        j->nc[k] = (int)(d->l[k] / rcmax);
        if (j->nc[k] < 1)
        {
            delete j;
            return fmdg_set_error("fmdg_srv_submit: box shorter than the cutoff");
        }
        j->cellh[k] = d->l[k] / j->nc[k];
    }
    j->nkinds = d->nkinds;
    for (int k = 0; k < d->nkinds; k++)
    {
        j->mass[k] = d->mass[k];
        j->elem[k] = d->eam_elem ? d->eam_elem[k] : -1;
    }
    j->eam_key = d->eam_key;
    j->n = d->n;
    j->x.assign(d->x, d->x + 3 * (size_t)d->n);
    j->v.assign(d->v, d->v + 3 * (size_t)d->n);
    j->kind.assign(d->kind, d->kind + d->n);
    for (int a = 0; a < d->n; a++)
        if (j->kind[a] >= (unsigned)d->nkinds)
        {
            delete j;
            return fmdg_set_error("fmdg_srv_submit: atom kind out of range");
        }
    j->steps = d->steps;
    j->dt = d->dt;
    j->prec = d->precision;
    j->keep_state = d->keep_state;
    // host binning: floor(x/cellh) per axis, input order inside a cell
    const int ncell = j->nc[0] * j->nc[1] * j->nc[2];
    j->cell_count.assign(ncell, 0);
    std::vector<int> cell(d->n);
    for (int a = 0; a < d->n; a++)
    {
        int c3[3];
        for (int k = 0; k < 3; k++)
        {
            const double q = floor(j->x[3 * (size_t)a + k] / j->cellh[k]);
            if (!(q >= 0.0 && q < j->nc[k]))
            {
                delete j;
                return fmdg_set_error("fmdg_srv_submit: atom outside the box");
            }
            c3[k] = (int)q;
        }
        cell[a] = c3[2] + j->nc[2] * (c3[1] + j->nc[1] * c3[0]);
        j->cell_count[cell[a]]++;
    }
    std::vector<int> start(ncell + 1, 0);
    for (int c = 0; c < ncell; c++) start[c + 1] = start[c] + j->cell_count[c];
    j->order.resize(d->n);
    for (int a = 0; a < d->n; a++) j->order[start[cell[a]]++] = a;
    // device bytes, with the list capacity the system will get
    const int maxnb = j->list_capacity > 0 ? j->list_capacity
                                           : fmdg_capacity_estimate(j->cell_count.data(), ncell,
                                                                    j->cellh[0] * j->cellh[1] * j->cellh[2], rl);
    j->bytes = fmdg_bytes_estimate(d->n, ncell, maxnb);
    j->id = S->next_id++;
    j->t_submit = wall_s() - S->t0;
    S->jobs[j->id] = j;
    S->queue.push_back(j);
    *id = j->id;
    return FMDG_OK;
}

// One turn of the serving loop: finished chunks are reaped, queued jobs
// admitted, and every pack with work gets a new chunk while fewer than two
// are in flight.  wait=1 blocks on the oldest chunk when nothing new could
// be launched.
extern "C" int fmdg_srv_progress(fmdg_server_t *S, int wait, int *active)
{
    FMDG_CK(cudaSetDevice(S->device));
    int rc = FMDG_OK;
    each_pack(S, [&](Pack &p) { if (!rc) rc = reap(S, p, false); });
    if (rc) return rc;
    const size_t queued = S->queue.size();
    if ((rc = admit(S, 0.002))) return rc;
    const bool admitted = S->queue.size() != queued;
    bool launched = false;
    each_pack(S, [&](Pack &p) {
        if (rc || p.inflight.size() >= 2 || p.active() == 0) return;
        rc = launch_chunk(S, p);
        launched = true;
    });
    if (rc) return rc;
    if (wait && !launched && !admitted)
    {
        // the pack whose oldest chunk was launched first
        Pack *oldest = nullptr;
        each_pack(S, [&](Pack &p) {
            if (!p.inflight.empty() && (!oldest || p.inflight.front().seq < oldest->inflight.front().seq))
                oldest = &p;
        });
        if (oldest && (rc = reap(S, *oldest, true))) return rc;
    }
    if (active) *active = (int)S->queue.size() + S->running;
    return FMDG_OK;
}

extern "C" int fmdg_srv_result(fmdg_server_t *S, long long id, fmdg_job_result_t *out)
{
    auto it = S->jobs.find(id);
    if (it == S->jobs.end()) return fmdg_set_error("fmdg_srv_result: unknown job");
    const Job *j = it->second;
    memset(out, 0, sizeof *out);
    out->state = j->state;
    out->error = j->fail_code;
    out->n = j->n;
    out->steps = j->steps;
    out->t_submit = j->t_submit;
    out->t_start = j->t_start;
    out->t_done = j->t_done;
    out->first = j->th0;
    out->last = j->th1;
    out->errbits = j->errs;
    out->device_bytes = (double)j->bytes;
    return FMDG_OK;
}

extern "C" int fmdg_srv_state(fmdg_server_t *S, long long id, double *x, double *v, double *F, unsigned *atomid)
{
    auto it = S->jobs.find(id);
    if (it == S->jobs.end()) return fmdg_set_error("fmdg_srv_state: unknown job");
    const Job *j = it->second;
    if (j->state != JOB_DONE || !j->keep_state) return FMDG_E_STATE;
    const size_t n = j->fid.size();
    if (x) memcpy(x, j->fx.data(), 3 * n * 8);
    if (v) memcpy(v, j->fv.data(), 3 * n * 8);
    if (F) memcpy(F, j->fF.data(), 3 * n * 8);
    if (atomid) memcpy(atomid, j->fid.data(), n * 4);
    return FMDG_OK;
}

extern "C" int fmdg_srv_release(fmdg_server_t *S, long long id)
{
    auto it = S->jobs.find(id);
    if (it == S->jobs.end()) return fmdg_set_error("fmdg_srv_release: unknown job");
    Job *j = it->second;
    if (j->state != JOB_DONE && j->state != JOB_FAILED) return FMDG_E_STATE;
    delete j;
    S->jobs.erase(it);
    return FMDG_OK;
}

extern "C" int fmdg_srv_now(fmdg_server_t *S, double *t)
{
    *t = wall_s() - S->t0;
    return FMDG_OK;
}

extern "C" int fmdg_srv_stats(fmdg_server_t *S, fmdg_srv_stats_t *out)
{
    memset(out, 0, sizeof *out);
    out->queued = (int)S->queue.size();
    out->running = S->running;
    out->admitted = S->admitted;
    out->finished = S->finished;
    out->failed = S->failed;
    out->atom_steps = S->atom_steps_done;
    out->kernels = S->kernels;
    out->bytes_in_use = (double)S->used;
    out->bytes_peak = (double)S->peak;
    for (int c = 0; c < 4; c++)
        for (int m = 0; m < 2; m++)
        {
            const Tuner &t = S->tuners[c][m];
            out->pack_fblk[c][m] = S->fixed_fblk ? S->fixed_fblk : (t.tuned ? t.fblk : 0);
            for (const Pack *p : S->packs[c][m])
            {
                out->pack_chunks[c][m] += p->chunks;
                out->pack_rebuilds[c][m] += p->rebuilds;
            }
        }
    return FMDG_OK;
}

// Admit every queued job that fits now (no steps launched).
extern "C" int fmdg_srv_admit(fmdg_server_t *S)
{
    FMDG_CK(cudaSetDevice(S->device));
    return admit(S, 0.0);
}

// Advance every admitted job by k chunks: the packs' chunk graphs are
// replayed on their streams, which start together after an event on a
// join stream; *ms is the device time from that event until every pack
// has finished (events on the join stream).  Every member needs at least
// k * chunk_steps steps left.
extern "C" int fmdg_srv_run_resident(fmdg_server_t *S, int k, float *ms)
{
    FMDG_CK(cudaSetDevice(S->device));
    if (!S->join)
    {
        FMDG_CK(cudaStreamCreateWithFlags(&S->join, cudaStreamNonBlocking));
        FMDG_CK(cudaEventCreate(&S->jev0));
        FMDG_CK(cudaEventCreate(&S->jev1));
    }
    int rc = FMDG_OK;
    each_pack(S, [&](Pack &p) {
        for (Job *j : p.members)
            if (!rc && j->left < k * S->chunk) rc = fmdg_set_error("fmdg_srv_run_resident: a job has too few steps left");
        if (p.exec && p.exec_fblk != want_fblk(S, p)) p.dirty = true;
        if (!rc && p.dirty) rc = rebuild(S, p);
    });
    if (rc) return rc;
    FMDG_CK(cudaEventRecord(S->jev0, S->join));
    std::vector<cudaEvent_t> ends;
    each_pack(S, [&](Pack &p) {
        if (rc || p.members.empty() || !p.exec) return;
        if (cudaStreamWaitEvent(p.stream, S->jev0, 0) != cudaSuccess) rc = fmdg_set_error("stream wait");
        for (int q = 0; q < k && !rc; q++) rc = launch_chunk(S, p);
        if (!rc) ends.push_back(p.inflight.back().ev1);
    });
    if (rc) return rc;
    for (cudaEvent_t e : ends) FMDG_CK(cudaStreamWaitEvent(S->join, e, 0));
    FMDG_CK(cudaEventRecord(S->jev1, S->join));
    FMDG_CK(cudaEventSynchronize(S->jev1));
    FMDG_CK(cudaEventElapsedTime(ms, S->jev0, S->jev1));
    each_pack(S, [&](Pack &p) { if (!rc) rc = reap(S, p, false); });
    return rc;
}

// One step of the pack (category, precision) launched phase by phase
// between events on its stream (no graph): ms[0] refresh, ms[1] neighbour
// lists, ms[2] EAM density, ms[3] pair forces + finish step; *atoms = the
// pack's atoms, *members = its jobs.
extern "C" int fmdg_srv_profile_pack(fmdg_server_t *S, int cls, int mixed, float ms[4], double *atoms,
                                     int *members)
{
    FMDG_CK(cudaSetDevice(S->device));
    if (cls < 0 || cls > 3 || mixed < 0 || mixed > 1) return fmdg_set_error("fmdg_srv_profile_pack: bad pack");
    *atoms = 0.0;
    *members = 0;
    for (int q = 0; q < 4; q++) ms[q] = 0.f;
    for (Pack *pp : S->packs[cls][mixed])
    {
        Pack &p = *pp;
        int rc;
        if (p.exec && p.exec_fblk != want_fblk(S, p)) p.dirty = true;
        if (p.dirty && (rc = rebuild(S, p))) return rc;
        if (p.members.empty()) continue;
        for (Job *j : p.members)
            if (j->left < 1) return fmdg_set_error("fmdg_srv_profile_pack: a job has no step left");
        // the pack's earlier chunks first
        FMDG_CK(cudaStreamSynchronize(p.stream));
        cudaEvent_t ev[5];
        for (int q = 0; q < 5; q++) ev[q] = get_event(S);
        FMDG_CK(cudaEventRecord(ev[0], p.stream));
        int n = fmdg_pack_launch_refresh(p.P);
        if (n < 0) return -n;
        S->kernels += n;
        FMDG_CK(cudaEventRecord(ev[1], p.stream));
        const int masks[3] = {1, 2, 4};
        for (int q = 0; q < 3; q++)
        {
            n = fmdg_pack_launch_forces(p.P, masks[q]);
            if (n < 0) return -n;
            S->kernels += n;
            FMDG_CK(cudaEventRecord(ev[q + 2], p.stream));
        }
        FMDG_CK(cudaEventSynchronize(ev[4]));
        for (int q = 0; q < 4; q++)
        {
            float t = 0.f;
            FMDG_CK(cudaEventElapsedTime(&t, ev[q], ev[q + 1]));
            ms[q] += t;
        }
        for (int q = 0; q < 5; q++) put_event(S, ev[q]);
        *members += (int)p.members.size();
        double a = 0.0;
        for (Job *j : p.members)
        {
            j->left -= 1;
            a += j->n;
            if (j->left == 0) p.dirty = true;
        }
        *atoms += a;
        S->atom_steps_done += a;
    }
    return FMDG_OK;
}
