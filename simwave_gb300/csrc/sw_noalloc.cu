// sw_noalloc.cu -- simwave_forward_device_noalloc: the float32 3D forward on
// caller-owned device arrays without any device allocation by this library.
//
// Who needs it: callers that must not (or cannot) allocate device memory
// while they run us -- a host framework that owns the whole device memory
// budget through its own pool and forbids allocations behind its back, or a
// latency-critical serving loop where cudaMalloc/cudaFree would synchronise
// the device and stall other work. The regular device entry keeps its
// scratch (per-point coefficient grids, a few status words) in buffers it
// allocates on first use; this entry keeps the same scratch in one
// file-scope device array of fixed size instead.
//
// Limits and behaviour:
//   * scratch is SIMWAVE_NOALLOC_SCRATCH_BYTES (32 MiB) per GPU that loads
//     the library, held until the process exits: 8 bytes per grid point
//     (two float coefficient grids) plus 256 bytes of status words, so grids
//     of up to (32 MiB - 256 B) / 8 points (pitched layout) are accepted;
//     larger grids are refused with SIMWAVE_E_ARGUMENT and a message;
//   * float32, 3D only (the tiled stencil); the layout must suit the tiled
//     kernel (pitch a multiple of 4 elements, lead + r a multiple of 32,
//     16-byte aligned arrays: what simwave_layout() returns), otherwise the
//     call is refused;
//   * flags: only SIMWAVE_FLAG_WINDOWS_CHECKED is honoured; every other flag
//     (timing events, the generic kernel, per-step launches) is refused;
//   * the call must not be made on a stream that is being captured into a
//     CUDA graph: it reads the zero-box bounds and the status word back to
//     the host and waits for its stream mid-call, which capture forbids, so
//     a capturing stream is refused up front (the capture stays intact);
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (that device current);
//   * the stencil is the one the regular entry runs, except where that one
//     would read the density's z derivative from a grid formed once per run
//     (it cannot be held in this scratch): the packed kernel then takes it
//     from its shared-memory queue instead -- same operator;
//   * every call shares the one array: the status words are cleared at the
//     start of each call, and calls that overlap on the GPU (from several
//     host threads or streams at once) race on it -- serialise them.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "simwave_gb300.h"
#include "sw_kernels.cuh"
#include "sw_tiled.h"

namespace sw {
namespace noalloc {

constexpr size_t kScratchBytes = SIMWAVE_NOALLOC_SCRATCH_BYTES;
constexpr size_t kWordsBytes = 256;  // zero box [0, 7), status word [7]

// The scratch: status words, then the C and Q coefficient grids.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct Refusal {
    int code;
    std::string message;
};

[[noreturn]] static void refuse(int code, const std::string& m) { throw Refusal{code, m}; }

#define NA_CUDA(expr)                                                             \
    do {                                                                          \
        cudaError_t e_ = (expr);                                                  \
        if (e_ != cudaSuccess)                                                    \
            refuse(SIMWAVE_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device address of g_scratch, looked up once per device with that device
// current (the host-side name is only a stand-in, not a device address).
static unsigned char* scratch_address() {
    static std::mutex m;
    static void* addr[64] = {};
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) refuse(SIMWAVE_E_ARGUMENT, "device index out of range");
    std::lock_guard<std::mutex> lock(m);
    if (!addr[dev]) {
        void* p = nullptr;
        NA_CUDA(cudaGetSymbolAddress(&p, g_scratch));
        addr[dev] = p;
    }
    return static_cast<unsigned char*>(addr[dev]);
}

// Exchange the contents of two equal-sized device regions in place.
__global__ void swap_regions(float* __restrict__ a, float* __restrict__ b, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float t = a[i];
        a[i] = b[i];
        b[i] = t;
    }
}

struct Slots {
    int prev, cur, next;
};

// The reference's time-level slot bookkeeping (constant_density/2d/wave.c:
// 110-122, 466-514), with the even-stride exchange kept as a relabelling of
// physical slots (perm[logical] = physical).
static std::vector<Slots> slot_schedule(size_t begin, size_t end, size_t stride,
                                        size_t nslots, std::vector<int>& perm) {
    std::vector<Slots> steps;
    perm.resize(nslots);
    for (size_t i = 0; i < nslots; i++) perm[i] = (int)i;
    size_t prev = 0, cur = 1, next = 2;
    for (size_t n = begin; n <= end; n++) {
        if (stride == 0) {
            prev = (n - 1) % 3;
            cur = n % 3;
            next = (n + 1) % 3;
        } else if (stride == 1) {
            prev = n - 1;
            cur = n;
            next = n + 1;
        }
        if (prev >= nslots || cur >= nslots || next >= nslots)
            refuse(SIMWAVE_E_SCHEDULE, "time step " + std::to_string(n) +
                                           " needs more wavefield slots than num_snapshots");
        steps.push_back({perm[prev], perm[cur], perm[next]});
        if (stride > 1) {
            if (n % stride == 1) {
                prev = cur;
                cur += 1;
                next += 1;
                if (stride % 2 == 0 && n < end) {
                    std::swap(cur, next);
                    if (cur >= nslots || next >= nslots)
                        refuse(SIMWAVE_E_SCHEDULE, "even-stride exchange needs more slots");
                    std::swap(perm[cur], perm[next]);
                }
            } else {
                prev = cur;
                cur = next;
                next = prev;
            }
        }
    }
    return steps;
}

static void check_windows(const char* what, const size_t* div, const size_t* doff,
                          size_t values_size, size_t count, const size_t ext[3],
                          cudaStream_t st) {
    if (!count) return;
    if (!div || !doff) refuse(SIMWAVE_E_ARGUMENT, std::string(what) + " arrays missing");
    std::vector<size_t> iv(count * 6), off(count);
    NA_CUDA(cudaMemcpyAsync(iv.data(), div, iv.size() * sizeof(size_t), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaMemcpyAsync(off.data(), doff, off.size() * sizeof(size_t), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    for (size_t s = 0; s < count; s++) {
        size_t len = 0;
        for (int a = 0; a < 3; a++) {
            const size_t b = iv[6 * s + 2 * a], e = iv[6 * s + 2 * a + 1];
            if (b > e || e >= ext[a])
                refuse(SIMWAVE_E_ARGUMENT, std::string(what) + " window outside the grid");
            len += e - b + 1;
        }
        if (off[s] > values_size || len > values_size - off[s])
            refuse(SIMWAVE_E_ARGUMENT, std::string(what) + " values offset out of range");
    }
}

static int run(const simwave_problem* P, cudaStream_t st) {
    if (!P) refuse(SIMWAVE_E_ARGUMENT, "null problem");
    if (P->dim != 3 || P->precision != 4)
        refuse(SIMWAVE_E_ARGUMENT, "the allocation-free entry runs 3D float32 problems only");
    if (P->flags & SIMWAVE_FLAG_TIME_KERNELS)
        refuse(SIMWAVE_E_ARGUMENT, "SIMWAVE_FLAG_TIME_KERNELS is not available without allocation");
    if (P->flags & ~SIMWAVE_FLAG_WINDOWS_CHECKED)
        refuse(SIMWAVE_E_ARGUMENT,
               "the allocation-free entry honours only SIMWAVE_FLAG_WINDOWS_CHECKED");
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        NA_CUDA(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            refuse(SIMWAVE_E_ARGUMENT,
                   "the allocation-free entry waits for its stream mid-call and cannot run "
                   "on a stream that is being captured");
    }
    if (P->space_order < 2 || P->space_order > 20 || P->space_order % 2)
        refuse(SIMWAVE_E_ARGUMENT, "space_order must be even in 2..20");
    const int r = P->space_order / 2;
    if (P->nz < (size_t)(2 * r + 1) || P->nx < (size_t)(2 * r + 1) || P->ny < (size_t)(2 * r + 1))
        refuse(SIMWAVE_E_ARGUMENT, "every grid extent must be >= space_order + 1");
    if (P->pitch < P->lead + P->ny) refuse(SIMWAVE_E_ARGUMENT, "pitch < lead + ny");
    const bool vd = P->variable_density != 0;
    if (!P->u || !P->velocity || !P->damp || (vd && (!P->density || !P->coeff_order1)) ||
        !P->coeff_order2 || !P->boundary_conditions || (P->num_receivers && !P->receivers) ||
        (P->num_sources && !P->wavelet))
        refuse(SIMWAVE_E_ARGUMENT, "null array argument");
    for (int e = 0; e < 6; e++)
        if (P->boundary_conditions[e] > 2)
            refuse(SIMWAVE_E_ARGUMENT, "boundary code must be 0, 1 or 2");
    // elements of one pitched grid, each product checked before it is formed;
    // the scratch also holds three per-axis tables of the damping mask
    const size_t tables = P->nz + P->nx + P->ny + 32;
    if (tables > (kScratchBytes - kWordsBytes) / sizeof(float))
        refuse(SIMWAVE_E_ARGUMENT, "grid extents exceed the allocation-free scratch");
    const size_t capacity =
        ((kScratchBytes - kWordsBytes) / sizeof(float) - tables) / 2;
    if (P->pitch > capacity || P->nx > capacity / P->pitch ||
        P->nz > capacity / (P->nx * P->pitch))
        refuse(SIMWAVE_E_ARGUMENT,
               "grid of " + std::to_string(P->nz) + " x " + std::to_string(P->nx) + " x " +
                   std::to_string(P->pitch) + " pitched points exceeds the " +
                   "allocation-free scratch (" + std::to_string(capacity) + " points)");
    const size_t grid = P->nz * P->nx * P->pitch;
    if (P->num_snapshots > 1 && P->slot_stride < grid)
        refuse(SIMWAVE_E_ARGUMENT, "slot_stride smaller than one grid");
    if (P->begin_timestep < 1) refuse(SIMWAVE_E_ARGUMENT, "begin_timestep must be >= 1");
    if (P->num_sources && P->end_timestep >= P->begin_timestep) {
        const size_t need = P->wavelet_count > 1 ? P->end_timestep * P->num_sources
                                                 : P->end_timestep;
        if (P->wavelet_size * (P->wavelet_count ? P->wavelet_count : 1) < need)
            refuse(SIMWAVE_E_ARGUMENT, "wavelet shorter than end_timestep");
    }
    const size_t ext[3] = {P->nz, P->nx, P->ny};
    if (!(P->flags & SIMWAVE_FLAG_WINDOWS_CHECKED)) {
        check_windows("src", P->src_points_interval, P->src_points_values_offset,
                      P->src_points_values_size, P->num_sources, ext, st);
        check_windows("rec", P->rec_points_interval, P->rec_points_values_offset,
                      P->rec_points_values_size, P->num_receivers, ext, st);
    }
    std::vector<int> perm;
    const std::vector<Slots> steps = slot_schedule(P->begin_timestep, P->end_timestep,
                                                   P->saving_stride, P->num_snapshots, perm);

    Layout L;
    L.dim = 3;
    L.r = r;
    L.nz = (long long)P->nz;
    L.nx = (long long)P->nx;
    L.ny = (long long)P->ny;
    L.pitch = (long long)P->pitch;
    L.lead = (long long)P->lead;
    L.plane = L.nx * L.pitch;
    L.slot = (long long)P->slot_stride;
    float* u = (float*)P->u;
    const float* vel = (const float*)P->velocity;
    const float* den = (const float*)P->density;
    const float* damp = (const float*)P->damp;

    TiledContext ctx;
    if (!tiled_prepare(ctx, L, vd, u, (long long)P->num_snapshots, L.slot, den))
        refuse(SIMWAVE_E_ARGUMENT,
               "layout not usable by the tiled kernel (use simwave_layout(): pitch a "
               "multiple of 4, lead + r a multiple of 32, arrays 16-byte aligned)");

    // scratch: words (zero box [0, 7), status [7], damping-table check [8]),
    // then C, Q and the per-axis damping tables; clear the previous call's words
    unsigned char* base = scratch_address();
    int* words = reinterpret_cast<int*>(base);
    float* C = reinterpret_cast<float*>(base + kWordsBytes);
    float* Q = C + grid;
    float* tabs = Q + grid;
    NA_CUDA(cudaMemsetAsync(words, 0, kWordsBytes, st));
    form_coefficients(vel, damp, C, Q, (long long)grid, (float)P->dt, st);
    NA_CUDA(cudaGetLastError());
    find_zero_box(Q, L, words, st);
    NA_CUDA(cudaGetLastError());
    if (ctx.tm && ctx.tm_tables) {
        damp_face_tables(damp, L, words, tabs, tabs + L.nz, tabs + L.nz + L.nx, words + 8, st);
        NA_CUDA(cudaGetLastError());
    }
    int box[9];
    NA_CUDA(cudaMemcpyAsync(box, words, sizeof(box), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    const bool good = box[6] == 0 && box[1] > box[0] && box[3] > box[2] && box[5] > box[4];
    for (int i = 0; i < 6; i++) ctx.zero_box[i] = good ? box[i] : 0;
    if (ctx.tm && ctx.tm_tables) {
        ctx.damp = damp;
        ctx.damp_tz = tabs;
        ctx.damp_tx = tabs + L.nz;
        ctx.damp_ty = tabs + L.nz + L.nx;
        ctx.damp_faces_ok = good && box[8] == 0;
        ctx.inv_dt = (float)(1.0 / P->dt);
    }
    ctx.err = words + 7;
    ctx.coefC = C;
    ctx.coefQ = Q;

    // weights: unscaled half weights, per-axis 1/h^2 and 1/(4 h^2)
    const Weights<float> W = make_weights<float>(
        (const float*)P->coeff_order2, vd ? (const float*)P->coeff_order1 : nullptr, r,
        P->dz, P->dx, P->dy);
    const float dt = (float)P->dt, dt2 = dt * dt;
    int bc[6];
    for (int e = 0; e < 6; e++) bc[e] = (int)P->boundary_conditions[e];
    Windows<float> src{P->src_points_interval, (const float*)P->src_points_values,
                       P->src_points_values_offset, P->num_sources};
    Windows<float> rec{P->rec_points_interval, (const float*)P->rec_points_values,
                       P->rec_points_values_offset, P->num_receivers};
    float* receivers = (float*)P->receivers;

    const int phases[3] = {2, 1, 0};  // y, x, z edges, the reference's order
    for (size_t i = 0; i < steps.size(); i++) {
        const size_t n = P->begin_timestep + i;
        float* un = u + (size_t)steps[i].next * L.slot;
        const float* uc = u + (size_t)steps[i].cur * L.slot;
        const float* up = u + (size_t)steps[i].prev * L.slot;
        tiled_launch(ctx, vd, un, uc, up, C, den, Q, L, W, dt, dt2, st);
        NA_CUDA(cudaGetLastError());
        if (src.count) {
            inject_sources<float, 3><<<(unsigned)src.count, 128, 0, st>>>(
                un, vel, damp, L, src, (const float*)P->wavelet, P->wavelet_count, n, dt, dt2);
            NA_CUDA(cudaGetLastError());
        }
        for (int ph = 0; ph < 3; ph++) {
            const int a = phases[ph];
            if (!bc[2 * a] && !bc[2 * a + 1]) continue;
            const int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
            const long long lines = (L.extent(a1) - 2 * r) * (L.extent(a2) - 2 * r);
            boundary_phase<float><<<(unsigned)((lines + 255) / 256), 256, 0, st>>>(
                un, L, a, bc[2 * a], bc[2 * a + 1]);
            NA_CUDA(cudaGetLastError());
        }
        if (rec.count) {
            const size_t threads = rec.count * 32;
            record_receivers<float, 3><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                receivers + (n - 1) * rec.count, uc, L, rec);
            NA_CUDA(cudaGetLastError());
        }
    }
    // undo the relabelling of the even-stride exchanges with in-place swaps
    // (cycle by cycle), so logical slot j ends in slot j as in the reference
    const int nslots = (int)P->num_snapshots;
    std::vector<int> at(nslots), where(nslots);  // at[physical] = logical content
    for (int j = 0; j < nslots; j++) {
        at[perm[j]] = j;
        where[j] = perm[j];
    }
    for (int j = 0; j < nslots; j++) {
        const int p = where[j];
        if (p == j) continue;
        swap_regions<<<1024, 256, 0, st>>>(u + (size_t)j * L.slot, u + (size_t)p * L.slot,
                                           (long long)grid);
        NA_CUDA(cudaGetLastError());
        const int other = at[j];  // logical content that sat in slot j
        at[p] = other;
        where[other] = p;
        at[j] = j;
        where[j] = j;
    }
    int code = 0;
    NA_CUDA(cudaMemcpyAsync(&code, words + 7, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    if (code) refuse(code, "a device wait gave up (bounded mbarrier wait expired)");
    return SIMWAVE_OK;
}

}  // namespace noalloc

// message for simwave_last_error() (sw_forward.cu)
void record_error(const std::string& message);

}  // namespace sw

extern "C" int simwave_forward_device_noalloc(const simwave_problem* problem, void* stream) {
    try {
        sw::record_error("");
        return sw::noalloc::run(problem, (cudaStream_t)stream);
    } catch (const sw::noalloc::Refusal& r) {
        sw::record_error(r.message);
        return r.code;
    } catch (const std::exception& e) {
        sw::record_error(e.what());
        return SIMWAVE_E_ARGUMENT;
    }
}
