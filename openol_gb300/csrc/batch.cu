// batch.cu -- many propagations of uneven sizes, methods and wavelengths in
// one persistent launch (olg_batch_*).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "propk.cuh"

using namespace olg;

// Many propagations of uneven sizes, methods and wavelengths in one launch.
// Work items, in queue order: every chirp job, then every pass-1 row group,
// every pass-2 column tile, every pass-3 row group (large fields first within
// each pass).  A CTA (one per SM, 512 threads) takes the next item with an
// atomic ticket, waits until the item's field has finished the pass it depends
// on (per-field counters; the wait is bounded and only ever on items taken
// earlier by running CTAs, so it cannot deadlock), runs it with the same pass
// bodies as the single-call kernels, then publishes its completion.
namespace olg {

constexpr int BATCH_NT = 512;
constexpr int BATCH_CTAS_PER_SM = 1;
// rows per row unit and columns per column tile: 16384 elements per unit
// (two 8192-point columns, as the fastest single-call column shape)
constexpr int BATCH_TILE = 2 * FFT_MAX;
__host__ __device__ constexpr int brow_nseq(int N) { return BATCH_TILE / N; }
__host__ __device__ constexpr int bcol_c(int N) { return BATCH_TILE / N; }
constexpr int BATCH_SMEM = padded_len(FFT_MAX) * 2 * 8; // the largest pass tile

enum : int { BK_CHIRP = 0, BK_FWD = 1, BK_COLS = 2, BK_INV = 3 };

struct BatchItem {
    int field, kind, unit, n; // n: FFT length that selects the instantiation
    int count;                // consecutive units processed by this item
};
constexpr int BATCH_UNITS_PER_ITEM = 8; // 8 x 16384 elements per item

struct BatchDev {
    const PropParams *P;
    const ChirpAxis *jobs;
    const BatchItem *items;
    int n_items;
    int *head;
    int *done;         // per field: chirp jobs, pass-1 units, pass-2 units finished
    const int *target; // per field: how many of each there are
    int *err;
    long long wait;    // budget of one bounded wait, SM clock cycles
};

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool wait_at_least(const int *p, int target, long long budget)
{
    const long long t0 = clock64();
    while (ld_acquire(p) < target) {
        __nanosleep(100);
        if (clock64() - t0 > budget) return false;
    }
    return true;
}

template <int N>
__device__ __forceinline__ void batch_run(const PropParams &P, const ChirpAxis *jobs, const BatchItem &I, float2 *sm,
                                          int tid)
{
    if (I.kind == BK_CHIRP) {
        chirp_body<N, BATCH_NT>(jobs[I.unit >> 1], I.unit & 1, sm, tid);
    } else if (I.kind == BK_FWD) {
        rows_fwd_body<N, BATCH_NT, brow_nseq(N)>(P, I.unit * brow_nseq(N), sm, tid);
    } else if (I.kind == BK_COLS) {
        cols_body<N, BATCH_NT, bcol_c(N)>(P, I.unit * bcol_c(N), sm, tid);
    } else {
        float lsum = 0.f;
        rows_inv_body<N, BATCH_NT, brow_nseq(N)>(P, I.unit * brow_nseq(N), sm, tid, lsum);
    }
}

__global__ void __launch_bounds__(BATCH_NT, BATCH_CTAS_PER_SM) k_batch(BatchDev D)
{
    extern __shared__ float2 sm[];
    __shared__ int s_item, s_ok;
    __shared__ PropParams sP;
    const int tid = threadIdx.x;
    int loaded_field = -1;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(D.head, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= D.n_items) break;
        const BatchItem I = D.items[it];
        const int f = I.field;
        if (tid == 0) {
            bool ok = true;
            if (I.kind == BK_FWD) ok = wait_at_least(D.done + 3 * f, D.target[3 * f], D.wait);
            else if (I.kind == BK_COLS)
                ok = wait_at_least(D.done + 3 * f + 1, D.target[3 * f + 1], D.wait) &&
                     wait_at_least(D.done + 3 * f, D.target[3 * f], D.wait);
            else if (I.kind == BK_INV) ok = wait_at_least(D.done + 3 * f + 2, D.target[3 * f + 2], D.wait);
            if (!ok) atomicExch(D.err, 1);
            __threadfence();
            s_ok = ok;
        }
        if (f != loaded_field) {
            const int *src = reinterpret_cast<const int *>(D.P + f);
            int *dst = reinterpret_cast<int *>(&sP);
            for (int w = tid; w < (int)(sizeof(PropParams) / 4); w += BATCH_NT) dst[w] = src[w];
            loaded_field = f;
        }
        __syncthreads();
        if (s_ok) {
            for (int u = 0; u < I.count; ++u) {
                BatchItem J = I;
                J.unit = I.unit + u;
                switch (I.n) {
                case 512: batch_run<512>(sP, D.jobs, J, sm, tid); break;
                case 1024: batch_run<1024>(sP, D.jobs, J, sm, tid); break;
                case 2048: batch_run<2048>(sP, D.jobs, J, sm, tid); break;
                case 4096: batch_run<4096>(sP, D.jobs, J, sm, tid); break;
                case 8192: batch_run<8192>(sP, D.jobs, J, sm, tid); break;
                default: break;
                }
                __syncthreads();
            }
        }
        __syncthreads();
        if (tid == 0 && I.kind != BK_INV) {
            __threadfence();
            atomicAdd(D.done + 3 * f + (I.kind == BK_CHIRP ? 0 : I.kind == BK_FWD ? 1 : 2), I.count);
        }
    }
}

} // namespace olg

struct olg_batch_plan_s {
    int dev = 0, n = 0, n_items = 0, grid = 0;
    std::vector<olg_field> fields;
    std::vector<char> direct; // per field: run through the tuned per-field passes, not k_batch
    std::vector<size_t> ws_off;
    char *mem = nullptr;
    size_t bytes = 0;
    BatchDev D{};
    size_t counters_off = 0, counters_bytes = 0;
    // olg_batch_execute_host: copy streams and events, made on first use
    cudaStream_t s_in = nullptr, s_out = nullptr;
    std::vector<cudaEvent_t> ev; // entry, small inputs in, small done, out done, per field: in, computed
};

namespace olg {
namespace {

bool batch_size_ok(int n) { return n >= 256 && n <= FFT_MAX / 2 && is_pow2(n); }

// Fields of at least this many pixels leave the persistent kernel: each fills
// the GPU on its own, and the per-field passes (autotuned launch shapes, no
// register cap shared with the largest length) run them faster; the
// persistent launch keeps the many small fields, where launches would cost
// more than the work.
std::atomic<long long> g_batch_direct_pixels{2048LL * 2048LL};

// the physical checks of the single-call entry points, per method
int check_field(const olg_field &F)
{
    if (F.method < OLG_BATCH_ASM || F.method > OLG_BATCH_FRESNEL_BANDLIMIT)
        return fail(OLG_ERR_INVALID_ARG, "unknown propagation method");
    if (int rc = check_phys(F.dy, F.dx, F.lambda, F.z, F.method != OLG_BATCH_ASM)) return rc;
    if (F.method == OLG_BATCH_ARSS) {
        if (!std::isfinite(F.s) || !std::isfinite(F.oy) || !std::isfinite(F.ox))
            return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
        if (F.s == 0.0 || F.s == 1.0)
            return fail(OLG_ERR_INVALID_ARG, "ARSS is undefined for s = 0 or s = 1 (window limits divide by s|s-1|)");
    }
    return OLG_OK;
}

int field_setup(const olg_field &F, const Layout &L, PropSetup *S)
{
    switch (F.method) {
    case OLG_BATCH_ASM: return setup_asm(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, F.flags, L, S);
    case OLG_BATCH_FRESNEL: return setup_fresnel(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, 0, F.flags, L, S);
    case OLG_BATCH_FRESNEL_BANDLIMIT:
        return setup_fresnel(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, 1, F.flags, L, S);
    case OLG_BATCH_ARSS:
        return setup_arss(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, F.s, F.oy, F.ox, F.flags, L, S);
    default: return fail(OLG_ERR_INVALID_ARG, "unknown batch method");
    }
}

} // namespace
} // namespace olg

extern "C" int olg_batch_plan_create(const olg_field *fields, int n_fields, olg_batch_plan *out)
{
    if (!out || !fields || n_fields <= 0) return fail(OLG_ERR_INVALID_ARG, "no fields");
    *out = nullptr;
    for (int i = 0; i < n_fields; ++i) {
        const olg_field &F = fields[i];
        if (int rc = validate(F.in, F.out, F.ny, F.nx)) return rc;
        if (int rc = check_field(F)) return rc;
        if (!batch_size_ok(F.ny) || !batch_size_ok(F.nx))
            return fail(OLG_ERR_UNSUPPORTED_SIZE, "batched fields must be powers of two in [256, 4096]");
    }
    if (int rc = ensure_twiddles()) return rc;
    int dev = 0;
    if (cudaError_t e = cudaGetDevice(&dev); e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    auto *plan = new olg_batch_plan_s();
    plan->n = n_fields;
    plan->fields.assign(fields, fields + n_fields);
    plan->dev = dev;
    const long long direct_px = g_batch_direct_pixels.load();
    plan->direct.resize(n_fields);
    for (int i = 0; i < n_fields; ++i) plan->direct[i] = (long long)fields[i].ny * fields[i].nx >= direct_px;
    // device memory: [PropParams x n][ChirpAxis jobs][items][done 3n][target 3n][head, err][per-field scratch]
    std::vector<PropSetup> setups(n_fields);
    std::vector<ChirpAxis> jobs;
    std::vector<BatchItem> items;
    std::vector<int> target(3 * n_fields, 0);
    size_t o = 0;
    const size_t offP = o; o += align_up(sizeof(PropParams) * n_fields, 256);
    // at most two axes per field
    const size_t offJ = o; o += align_up(sizeof(ChirpAxis) * 2 * n_fields, 256);
    // item count: chirp <= 4 per field, rows and column tiles per field
    size_t n_items_max = 0;
    for (auto &F : plan->fields) {
        const int NX = 2 * F.nx, NY = 2 * F.ny;
        const int rows = (F.ny + brow_nseq(NX) - 1) / brow_nseq(NX);
        const int cols = (NX + bcol_c(NY) - 1) / bcol_c(NY);
        n_items_max += 4 + 2 * rows + cols;
    }
    const size_t offI = o; o += align_up(sizeof(BatchItem) * n_items_max, 256);
    const size_t offC = o; o += align_up(sizeof(int) * (6 * n_fields + 2), 256);
    plan->ws_off.resize(n_fields);
    for (int i = 0; i < n_fields; ++i) {
        plan->ws_off[i] = o;
        o += align_up(layout_bytes(plan->fields[i].ny, plan->fields[i].nx, nullptr, nullptr), 256);
    }
    plan->bytes = o;
    cudaError_t e = cudaMalloc(&plan->mem, plan->bytes);
    if (e != cudaSuccess) {
        delete plan;
        return cuda_fail(e, "cudaMalloc (batch plan)");
    }
    // per-field setup, chirp jobs and the item queue
    std::vector<int> order(n_fields);
    for (int i = 0; i < n_fields; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long)plan->fields[a].ny * plan->fields[a].nx > (long)plan->fields[b].ny * plan->fields[b].nx;
    });
    for (int i = 0; i < n_fields; ++i) {
        const olg_field &F = plan->fields[i];
        Layout L;
        layout_bytes(F.ny, F.nx, &L, plan->mem + plan->ws_off[i]);
        if (int rc = field_setup(F, L, &setups[i])) {
            cudaFree(plan->mem);
            delete plan;
            return rc;
        }
        setups[i].P.coherent = 1;
        if (setups[i].chirps && !plan->direct[i]) {
            for (int a = 0; a < 2; ++a) {
                const ChirpAxis &A = a ? setups[i].ay : setups[i].ax;
                const int jidx = (int)jobs.size();
                jobs.push_back(A);
                items.push_back({i, BK_CHIRP, 2 * jidx + 0, A.L, 1});
                target[3 * i] += 1;
                if (A.ta || A.tb) {
                    items.push_back({i, BK_CHIRP, 2 * jidx + 1, A.L, 1});
                    target[3 * i] += 1;
                }
            }
        }
    }
    for (int kind = BK_FWD; kind <= BK_INV; ++kind)
        for (int i : order) {
            if (plan->direct[i]) continue;
            const olg_field &F = plan->fields[i];
            const int NX = 2 * F.nx, NY = 2 * F.ny;
            if (kind == BK_COLS) {
                const int C = bcol_c(NY), units = (NX + C - 1) / C;
                for (int u = 0; u < units; u += BATCH_UNITS_PER_ITEM)
                    items.push_back({i, kind, u, NY, std::min(BATCH_UNITS_PER_ITEM, units - u)});
                target[3 * i + 2] = units;
            } else {
                const int R = brow_nseq(NX), units = (F.ny + R - 1) / R;
                for (int u = 0; u < units; u += BATCH_UNITS_PER_ITEM)
                    items.push_back({i, kind, u, NX, std::min(BATCH_UNITS_PER_ITEM, units - u)});
                if (kind == BK_FWD) target[3 * i + 1] = units;
            }
        }
    plan->n_items = (int)items.size();
    std::vector<PropParams> Ps(n_fields);
    for (int i = 0; i < n_fields; ++i) Ps[i] = setups[i].P;
    e = cudaMemcpy(plan->mem + offP, Ps.data(), sizeof(PropParams) * n_fields, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !jobs.empty())
        e = cudaMemcpy(plan->mem + offJ, jobs.data(), sizeof(ChirpAxis) * jobs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->mem + offI, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->mem + offC + sizeof(int) * 3 * n_fields, target.data(), sizeof(int) * 3 * n_fields,
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(plan->mem);
        delete plan;
        return cuda_fail(e, "uploading the batch plan");
    }
    int* C = (int *)(plan->mem + offC);
    plan->D.P = (const PropParams *)(plan->mem + offP);
    plan->D.jobs = (const ChirpAxis *)(plan->mem + offJ);
    plan->D.items = (const BatchItem *)(plan->mem + offI);
    plan->D.n_items = plan->n_items;
    plan->D.done = C;
    plan->D.target = C + 3 * n_fields;
    plan->D.head = C + 6 * n_fields;
    plan->D.err = C + 6 * n_fields + 1;
    plan->counters_off = offC;
    plan->counters_bytes = sizeof(int) * 3 * n_fields;
    plan->grid = sm_count() * BATCH_CTAS_PER_SM;
    e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, BATCH_SMEM);
    if (e != cudaSuccess) {
        cudaFree(plan->mem);
        delete plan;
        return cuda_fail(e, "cudaFuncSetAttribute(k_batch)");
    }
    *out = plan;
    return OLG_OK;
}

namespace olg {
namespace {

// one field through the single-field passes, in the plan's workspace
int batch_field_direct(olg_batch_plan plan, int i, cudaStream_t st)
{
    const olg_field &F = plan->fields[i];
    Layout L;
    layout_bytes(F.ny, F.nx, &L, plan->mem + plan->ws_off[i]);
    PropSetup S;
    if (int rc = field_setup(F, L, &S)) return rc;
    return run_setup(S, st);
}

} // namespace
} // namespace olg

extern "C" int olg_batch_execute(olg_batch_plan plan, olg_stream_t stream)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    // reset the done counters, the ticket and the error word (target stays)
    cudaError_t e = cudaMemsetAsync(plan->D.done, 0, plan->counters_bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(plan->D.head, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync (batch counters)");
    if (plan->n_items > 0) {
        plan->D.wait = wait_budget_cycles();
        k_batch<<<plan->grid, BATCH_NT, BATCH_SMEM, st>>>(plan->D);
        count_launch();
        if (int rc = check_launch("k_batch")) return rc;
    }
    for (int i = 0; i < plan->n; ++i)
        if (plan->direct[i])
            if (int rc = batch_field_direct(plan, i, st)) return rc;
    return OLG_OK;
}

namespace olg {
namespace {

int host_pipeline_init(olg_batch_plan plan)
{
    if (plan->s_in) return OLG_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&plan->s_in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&plan->s_out, cudaStreamNonBlocking);
    const int n_ev = 4 + 2 * plan->n;
    for (int i = 0; e == cudaSuccess && i < n_ev; ++i) {
        cudaEvent_t v = nullptr;
        e = cudaEventCreateWithFlags(&v, cudaEventDisableTiming);
        if (e == cudaSuccess) plan->ev.push_back(v);
    }
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "creating the batch copy streams");
}

int copy_field(void *dst, const void *src, const olg_field &F, cudaMemcpyKind kind, cudaStream_t st)
{
    const cudaError_t e = cudaMemcpyAsync(dst, src, sizeof(float2) * (size_t)F.ny * F.nx, kind, st);
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "cudaMemcpyAsync (batch field)");
}

} // namespace
} // namespace olg

// Host fields in and out, pipelined over three streams.  The copy-in stream
// brings every persistent-kernel field first, then the large fields one by
// one; the caller's stream runs the persistent launch as soon as its fields
// have arrived and each large field's passes as soon as that field has; the
// copy-out stream returns each result as soon as it is computed.  So the
// copies in, the propagations and the copies out overlap, and a step takes
// about the longest of the three instead of their sum.  Both copy streams
// first wait for the caller's stream, and the caller's stream waits for the
// last copy out, so the call is ordered on `stream` like olg_batch_execute.
extern "C" int olg_batch_execute_host(olg_batch_plan plan, const void *const *host_in, void *const *host_out,
                                      olg_stream_t stream)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    if (!host_in || !host_out) return fail(OLG_ERR_INVALID_ARG, "null host field arrays");
    for (int i = 0; i < plan->n; ++i)
        if (!host_in[i] || !host_out[i]) return fail(OLG_ERR_INVALID_ARG, "null host field");
    if (int rc = host_pipeline_init(plan)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t *ev = plan->ev.data();
    cudaEvent_t e_entry = ev[0], e_small_in = ev[1], e_small_done = ev[2], e_out_done = ev[3];
    cudaEvent_t *e_in = ev + 4, *e_done = ev + 4 + plan->n;
    auto ck = [](cudaError_t e, const char *what) { return e == cudaSuccess ? OLG_OK : cuda_fail(e, what); };
    if (int rc = ck(cudaEventRecord(e_entry, st), "cudaEventRecord")) return rc;
    if (int rc = ck(cudaStreamWaitEvent(plan->s_in, e_entry, 0), "cudaStreamWaitEvent")) return rc;
    if (int rc = ck(cudaStreamWaitEvent(plan->s_out, e_entry, 0), "cudaStreamWaitEvent")) return rc;
    // the persistent kernel's fields
    for (int i = 0; i < plan->n; ++i)
        if (!plan->direct[i])
            if (int rc = copy_field((void *)plan->fields[i].in, host_in[i], plan->fields[i], cudaMemcpyHostToDevice,
                                    plan->s_in))
                return rc;
    if (int rc = ck(cudaEventRecord(e_small_in, plan->s_in), "cudaEventRecord")) return rc;
    // the large fields, in order
    for (int i = 0; i < plan->n; ++i)
        if (plan->direct[i]) {
            if (int rc = copy_field((void *)plan->fields[i].in, host_in[i], plan->fields[i], cudaMemcpyHostToDevice,
                                    plan->s_in))
                return rc;
            if (int rc = ck(cudaEventRecord(e_in[i], plan->s_in), "cudaEventRecord")) return rc;
        }
    // compute on the caller's stream: the persistent launch, then each large field
    if (int rc = ck(cudaStreamWaitEvent(st, e_small_in, 0), "cudaStreamWaitEvent")) return rc;
    cudaError_t e = cudaMemsetAsync(plan->D.done, 0, plan->counters_bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(plan->D.head, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync (batch counters)");
    if (plan->n_items > 0) {
        plan->D.wait = wait_budget_cycles();
        k_batch<<<plan->grid, BATCH_NT, BATCH_SMEM, st>>>(plan->D);
        count_launch();
        if (int rc = check_launch("k_batch")) return rc;
    }
    if (int rc = ck(cudaEventRecord(e_small_done, st), "cudaEventRecord")) return rc;
    if (int rc = ck(cudaStreamWaitEvent(plan->s_out, e_small_done, 0), "cudaStreamWaitEvent")) return rc;
    for (int i = 0; i < plan->n; ++i)
        if (!plan->direct[i])
            if (int rc = copy_field(host_out[i], plan->fields[i].out, plan->fields[i], cudaMemcpyDeviceToHost,
                                    plan->s_out))
                return rc;
    for (int i = 0; i < plan->n; ++i)
        if (plan->direct[i]) {
            if (int rc = ck(cudaStreamWaitEvent(st, e_in[i], 0), "cudaStreamWaitEvent")) return rc;
            if (int rc = batch_field_direct(plan, i, st)) return rc;
            if (int rc = ck(cudaEventRecord(e_done[i], st), "cudaEventRecord")) return rc;
            if (int rc = ck(cudaStreamWaitEvent(plan->s_out, e_done[i], 0), "cudaStreamWaitEvent")) return rc;
            if (int rc = copy_field(host_out[i], plan->fields[i].out, plan->fields[i], cudaMemcpyDeviceToHost,
                                    plan->s_out))
                return rc;
        }
    // the caller's stream resumes after the last copy out (and the copy-in
    // stream has finished before the last computation, which waited on it)
    if (int rc = ck(cudaEventRecord(e_out_done, plan->s_out), "cudaEventRecord")) return rc;
    return ck(cudaStreamWaitEvent(st, e_out_done, 0), "cudaStreamWaitEvent");
}

extern "C" int olg_batch_execute_serial(olg_batch_plan plan, olg_stream_t stream)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    for (int i = 0; i < plan->n; ++i)
        if (int rc = batch_field_direct(plan, i, st)) return rc;
    return OLG_OK;
}

extern "C" long long olg_batch_direct_pixels(long long pixels)
{
    if (pixels > 0) return g_batch_direct_pixels.exchange(pixels);
    return g_batch_direct_pixels.load();
}

extern "C" int olg_batch_plan_direct_fields(olg_batch_plan plan)
{
    if (!plan) return 0;
    int n = 0;
    for (char d : plan->direct) n += d ? 1 : 0;
    return n;
}

extern "C" int olg_batch_check(olg_batch_plan plan)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    int err = 0;
    cudaError_t e = cudaMemcpy(&err, plan->D.err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "reading the batch error word");
    return err ? fail(OLG_ERR_CUDA, "a batched item gave up on a bounded wait") : OLG_OK;
}

extern "C" int olg_batch_plan_items(olg_batch_plan plan) { return plan ? plan->n_items : 0; }

extern "C" int olg_batch_plan_raise_target(olg_batch_plan plan, int field, int stage, int delta)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    if (field < 0 || field >= plan->n || stage < 0 || stage > 2 || delta < 0)
        return fail(OLG_ERR_INVALID_ARG, "field, stage (0..2) or delta (>= 0) out of range");
    int *t = const_cast<int *>(plan->D.target) + 3 * field + stage;
    int v = 0;
    cudaError_t e = cudaMemcpy(&v, t, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "reading a batch target");
    v += delta;
    e = cudaMemcpy(t, &v, sizeof(int), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "writing a batch target");
}

extern "C" int olg_batch_plan_destroy(olg_batch_plan plan)
{
    if (!plan) return OLG_OK;
    for (cudaEvent_t v : plan->ev) cudaEventDestroy(v);
    if (plan->s_in) cudaStreamDestroy(plan->s_in);
    if (plan->s_out) cudaStreamDestroy(plan->s_out);
    cudaError_t e = cudaFree(plan->mem);
    delete plan;
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "cudaFree (batch plan)");
}


// ------------------------------------------------- single-field plans
// One propagation's set-up done once: the parameters checked, the scratch
// (half-padded spectrum and chirp tables) allocated, and the Fresnel / ARSS
// chirp spectra computed; each execution binds the fields and runs the three
// passes.  Executions of one plan share its scratch, so they must be ordered
// (one stream, or synchronised between streams).
struct olg_prop_plan_s {
    olg_field F{};
    char *mem = nullptr;
    PropSetup S{};
    // olg_prop_plan_execute_host: three device field slots and the copy
    // pipeline, made on first use
    char *slots = nullptr;
    size_t slot_bytes = 0;
    HostPipeline pipe;
};

extern "C" int olg_prop_plan_create(const olg_field *field, olg_prop_plan *out)
{
    if (!out || !field) return fail(OLG_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    const olg_field &F = *field;
    if (!axis_ok(F.ny) || !axis_ok(F.nx))
        return fail(OLG_ERR_UNSUPPORTED_SIZE,
                    "ny, nx must be powers of two in [16, 4096] or have 2n = 2^a 3^b 5^c <= 7680 (n >= 8)");
    if (int rc = check_field(F)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    auto *plan = new olg_prop_plan_s();
    plan->F = F;
    const size_t bytes = layout_bytes(F.ny, F.nx, nullptr, nullptr);
    cudaError_t e = cudaMalloc(&plan->mem, bytes);
    if (e != cudaSuccess) {
        delete plan;
        return cuda_fail(e, "cudaMalloc (propagation plan)");
    }
    Layout L;
    layout_bytes(F.ny, F.nx, &L, plan->mem);
    olg_field G = F; // the fields are bound at execution; the scratch stands in
    G.in = plan->mem;
    G.out = plan->mem;
    int rc = field_setup(G, L, &plan->S);
    if (!rc && plan->S.chirps) {
        cudaStream_t st = nullptr;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate (propagation plan)");
        if (!rc) rc = chirp_axis(plan->S.ax, st);
        if (!rc) rc = chirp_axis(plan->S.ay, st);
        if (st) {
            e = cudaStreamSynchronize(st);
            if (!rc && e != cudaSuccess) rc = cuda_fail(e, "computing the plan's chirp spectra");
            cudaStreamDestroy(st);
        }
    }
    if (rc) {
        cudaFree(plan->mem);
        delete plan;
        return rc;
    }
    *out = plan;
    return OLG_OK;
}

extern "C" int olg_prop_plan_execute(olg_prop_plan plan, const void *in, void *out, olg_stream_t stream)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    if (int rc = validate(in, out, plan->F.ny, plan->F.nx)) return rc;
    PropParams P = plan->S.P;
    P.in = (const float2 *)in;
    P.out = (float2 *)out;
    return run_passes(P, (cudaStream_t)stream);
}

// A sequence of host fields through one plan: field i goes up into device
// slot i % 3 on the plan's copy-in stream, is propagated in place there on
// the caller's stream and comes down on the copy-out stream, so field i+1's
// copy in and field i-1's copy out overlap field i's passes.  Ordered on
// `stream` like `count` calls of olg_prop_plan_execute (the propagations
// themselves run one after another: they share the plan's scratch).
extern "C" int olg_prop_plan_execute_host(olg_prop_plan plan, const void *const *host_in, void *const *host_out,
                                          int count, olg_stream_t stream)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    if (count < 0) return fail(OLG_ERR_INVALID_ARG, "negative field count");
    if (count == 0) return OLG_OK;
    if (!host_in || !host_out) return fail(OLG_ERR_INVALID_ARG, "null host field arrays");
    for (int i = 0; i < count; ++i)
        if (!host_in[i] || !host_out[i]) return fail(OLG_ERR_INVALID_ARG, "null host field");
    const size_t field_bytes = sizeof(float2) * (size_t)plan->F.ny * plan->F.nx;
    if (!plan->slots) {
        const size_t sb = align_up(field_bytes, 256);
        const cudaError_t e = cudaMalloc(&plan->slots, HostPipeline::SLOTS * sb);
        if (e != cudaSuccess) {
            plan->slots = nullptr;
            return cuda_fail(e, "cudaMalloc (plan field slots)");
        }
        plan->slot_bytes = sb;
    }
    if (int rc = plan->pipe.init()) return rc;
    HostPipeline &H = plan->pipe;
    cudaStream_t st = (cudaStream_t)stream;
    auto enqueue = [&]() -> int {
        if (int rc = H.begin(st)) return rc;
        for (int i = 0; i < count; ++i) {
            char *dev = plan->slots + (size_t)(i % HostPipeline::SLOTS) * plan->slot_bytes;
            if (int rc = H.copy_in_begin(i)) return rc;
            cudaError_t e = cudaMemcpyAsync(dev, host_in[i], field_bytes, cudaMemcpyHostToDevice, H.s_in);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (field in)");
            if (int rc = H.copy_in_end(i, st)) return rc;
            PropParams P = plan->S.P;
            P.in = (const float2 *)dev;
            P.out = (float2 *)dev;
            if (int rc = run_passes(P, st)) return rc;
            if (int rc = H.compute_end(i, st)) return rc;
            e = cudaMemcpyAsync(host_out[i], dev, field_bytes, cudaMemcpyDeviceToHost, H.s_out);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (field out)");
            if (int rc = H.copy_out_end(i)) return rc;
        }
        return H.end(st);
    };
    const int rc = enqueue();
    // on a failure part way, the copies already queued finish before the
    // caller can reuse or free its host buffers
    if (rc) H.drain();
    return rc;
}

extern "C" int olg_prop_plan_destroy(olg_prop_plan plan)
{
    if (!plan) return OLG_OK;
    plan->pipe.release();
    cudaError_t e = cudaFree(plan->mem);
    if (plan->slots) {
        const cudaError_t e2 = cudaFree(plan->slots);
        if (e == cudaSuccess) e = e2;
    }
    delete plan;
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "cudaFree (propagation plan)");
}
