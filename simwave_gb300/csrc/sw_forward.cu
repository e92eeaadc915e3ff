// sw_forward.cu -- host driver and C ABI of libsimwave_gb300.so.
//
// Owns: argument validation, the time-level slot schedule, device buffers of
// the host-pointer entries, kernel launch sequence per time step, timing and
// error reporting. Kernels live in sw_kernels.cuh (generic) and
// sw_stencil_tiled.cu (tiled fast path).
#include <algorithm>
#include <atomic>
#include <type_traits>
#include <chrono>
#include <functional>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "simwave_gb300.h"
#include "sw_kernels.cuh"
#include "sw_tiled.h"

namespace sw {

// ---------------------------------------------------------------------------
// errors

struct Failure {
    int code;
    std::string message;
};

static thread_local std::string g_last_error;
static thread_local simwave_stats g_last_stats;

[[noreturn]] static void fail(int code, const std::string& msg) {
    throw Failure{code, msg};
}

// Sets the calling thread's simwave_last_error() message (for entry points
// defined in other translation units).
void record_error(const std::string& message) { g_last_error = message; }

#define SW_CUDA(expr)                                                       \
    do {                                                                    \
        cudaError_t e_ = (expr);                                            \
        if (e_ != cudaSuccess)                                              \
            ::sw::fail(e_ == cudaErrorMemoryAllocation ? SIMWAVE_E_MEMORY   \
                                                       : SIMWAVE_E_CUDA,    \
                       std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define SW_LAUNCHED(name)                                                   \
    do {                                                                    \
        cudaError_t e_ = cudaGetLastError();                                \
        if (e_ != cudaSuccess)                                              \
            ::sw::fail(SIMWAVE_E_CUDA,                                      \
                       std::string("launch ") + name + ": " +               \
                           cudaGetErrorString(e_));                         \
    } while (0)

// ---------------------------------------------------------------------------
// slot schedule
//
// The reference keeps every time level in a slot of `u` and moves three slot
// indices (prev, cur, next) per step (constant_density/2d/wave.c:110-122,
// 466-514): stride 0 rotates through slots 0..2, stride 1 writes level n+1
// into slot n+1, stride s > 1 advances one slot every s steps and, for even
// s, exchanges the contents of two slots. The schedule below replays that
// bookkeeping on the host. The exchange is realised as a relabelling of
// physical slots (perm), so no data moves; final contents of logical slot j
// are in physical slot perm[j].

struct StepSlots {
    int prev, cur, next;  // physical slots
};

struct Schedule {
    std::vector<StepSlots> steps;
    std::vector<int> perm;     // logical -> physical at the end
    std::vector<char> written; // physical slot written at least once
    std::vector<char> touched; // logical slot read or written
};

static Schedule make_schedule(size_t begin, size_t end, size_t stride,
                              size_t nslots) {
    Schedule S;
    S.perm.resize(nslots);
    for (size_t i = 0; i < nslots; i++) S.perm[i] = (int)i;
    S.written.assign(nslots, 0);
    S.touched.assign(nslots, 0);
    if (begin < 1) fail(SIMWAVE_E_ARGUMENT, "begin_timestep must be >= 1");
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
            fail(SIMWAVE_E_SCHEDULE,
                 "time step " + std::to_string(n) + " needs wavefield slot " +
                     std::to_string(std::max(prev, std::max(cur, next))) +
                     " but num_snapshots is " + std::to_string(nslots));
        S.steps.push_back({S.perm[prev], S.perm[cur], S.perm[next]});
        S.written[S.perm[next]] = 1;
        S.touched[prev] = S.touched[cur] = S.touched[next] = 1;
        if (stride > 1) {
            if (n % stride == 1) {
                prev = cur;
                cur += 1;
                next += 1;
                if (stride % 2 == 0 && n < end) {
                    std::swap(cur, next);
                    if (cur >= nslots || next >= nslots)
                        fail(SIMWAVE_E_SCHEDULE,
                             "even-stride exchange needs slot " +
                                 std::to_string(std::max(cur, next)) +
                                 " but num_snapshots is " +
                                 std::to_string(nslots));
                    std::swap(S.perm[cur], S.perm[next]);
                    S.touched[cur] = S.touched[next] = 1;
                }
            } else {
                prev = cur;
                cur = next;
                next = prev;
            }
        }
    }
    return S;
}

// ---------------------------------------------------------------------------
// layout

static void choose_layout(size_t nfast, int r, int precision, size_t* pitch,
                          size_t* lead) {
    const size_t align = 128 / (size_t)precision;  // elements per 128 B
    *lead = (align - (size_t)r % align) % align;
    *pitch = (*lead + nfast + align - 1) / align * align;
}

// ---------------------------------------------------------------------------
// device buffers owned by the host-pointer entries (grow-only, per device)

struct Buffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    void* ensure(size_t n) {
        if (n <= bytes) return ptr;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        if (n == 0) return nullptr;
        SW_CUDA(cudaMalloc(&ptr, n));
        SW_CUDA(cudaMemset(ptr, 0, n));  // row padding is never written
        // the memset runs on the legacy stream, which the library's
        // non-blocking streams do not wait for: finish it before any copy
        // into the buffer can be queued
        SW_CUDA(cudaDeviceSynchronize());
        bytes = n;
        return ptr;
    }
};

struct Arena {
    Buffer u, vel, den, damp, wavelet, rec;
    Buffer src_iv, src_val, src_off, rec_iv, rec_val, rec_off;
    Buffer scratch;
    Buffer stage_in[2], stage_out[2];  // dense staging of one grid each
    cudaStream_t stream = nullptr;     // time loop
    cudaStream_t copy_in = nullptr;    // host -> device copies and repacks
    cudaStream_t copy_out = nullptr;   // repacks and device -> host copies
    bool host_access = false;  // kernels may address pageable host memory
    std::vector<cudaEvent_t> events;
    cudaEvent_t event(size_t i) {
        while (events.size() <= i) {
            cudaEvent_t e;
            SW_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            events.push_back(e);
        }
        return events[i];
    }
};

static std::mutex g_mutex;  // serialises the host-pointer entries
static int g_transfer_mode = SIMWAVE_TRANSFER_AUTO;
static std::map<int, Arena> g_arenas;

static Arena& arena_for_current_device() {
    int dev = 0;
    SW_CUDA(cudaGetDevice(&dev));
    Arena& a = g_arenas[dev];
    if (!a.stream) SW_CUDA(cudaStreamCreateWithFlags(&a.stream, cudaStreamNonBlocking));
    if (!a.copy_in || !a.copy_out) {
        // copies at the highest priority: their repack kernels are small
        // (a read and a write of one grid) and get the next free block
        // slots, so a snapshot leaves while the time loop runs instead of
        // after it
        int lo = 0, hi = 0;
        SW_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        SW_CUDA(cudaStreamCreateWithPriority(&a.copy_in, cudaStreamNonBlocking, hi));
        SW_CUDA(cudaStreamCreateWithPriority(&a.copy_out, cudaStreamNonBlocking, hi));
        int pageable = 0;
        SW_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
        a.host_access = pageable != 0;
    }
    return a;
}

static std::mutex g_event_mutex;
static std::map<int, std::vector<cudaEvent_t>> g_event_pool;

// ---------------------------------------------------------------------------
// one forward run on device-resident data

template <typename T>
struct Run {
    Layout L;
    bool vd;
    T* u;
    size_t nslots;
    const T* vel;
    const T* den;
    const T* damp;
    const T* wavelet;
    size_t wavelet_count;
    Weights<T> W;
    int bc[6];
    Windows<T> src, rec;
    T* receivers;
    size_t begin, end, stride;
    T dt;
    unsigned flags;
    // optional hooks around each time step's launches (host-entry copies)
    std::function<void(size_t)> before_step, after_step;
};

template <typename T, int DIM, bool VD>
static void launch_stencil(const Run<T>& R, const TiledContext& tctx, T* un,
                           const T* uc, const T* up, cudaStream_t st,
                           int* variant, int* kernel) {
    const Layout& L = R.L;
    const T dt2 = R.dt * R.dt;
    if constexpr (std::is_same<T, float>::value && DIM == 2) {
        if (tctx.ok) {
            tiled2d_launch(L, VD, un, uc, up, tctx.coefC, tctx.coefQ, R.den, R.W,
                           tctx.zero_box, st);
            *variant = 1;
            SW_LAUNCHED("stencil2d_single");
            return;
        }
    }
    if constexpr (std::is_same<T, float>::value && DIM == 3) {
        if (tctx.ok) {
            *kernel = tiled_launch(tctx, VD, un, uc, up, tctx.coefC, R.den, tctx.coefQ, L,
                                   R.W, R.dt, dt2, st);
            *variant = 1;
            SW_LAUNCHED("stencil3d_tiled");
            return;
        }
    }
    const int r = L.r;
    dim3 block(32, 8, 1);
    dim3 grid((unsigned)((L.nfast() - 2 * r + 31) / 32),
              (unsigned)((L.nmid() - 2 * r + 7) / 8),
              DIM == 3 ? (unsigned)(L.nslow() - 2 * r) : 1u);
    stencil_generic<T, DIM, VD><<<grid, block, 0, st>>>(
        un, uc, up, R.vel, R.den, R.damp, L, R.W, R.dt, dt2);
    *variant = 0;
    SW_LAUNCHED("stencil_generic");
}

// Per-device words the kernels report into: [0..5] zero box, [6] box check,
// [7] error code of bounded waits. Allocated once per device.
static int* device_words() {
    static std::mutex m;
    static std::map<int, int*> words;
    int dev = 0;
    SW_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(m);
    int*& w = words[dev];
    if (!w) {
        SW_CUDA(cudaMalloc(&w, 16 * sizeof(int)));
        SW_CUDA(cudaMemset(w, 0, 16 * sizeof(int)));
        SW_CUDA(cudaDeviceSynchronize());  // zeroed before any stream reads it
    }
    return w;
}

// Tiled-kernel context of one run (float32): per-point coefficients C, Q and
// the zero-box words in scratch allocated on the run's stream (stream-ordered,
// so concurrent runs on different streams never share it), freed by
// release_tiled when the run's launches are queued.
template <typename T>
static TiledContext prepare_tiled(const Run<T>& R, cudaStream_t st) {
    TiledContext ctx;
    if constexpr (std::is_same<T, float>::value) {
        if (R.flags & SIMWAVE_FLAG_GENERIC_KERNEL) return ctx;
        const Layout& L = R.L;
        if (L.dim == 2) {
            if (!tiled2d_supported(L) ||
                (reinterpret_cast<uintptr_t>(R.u) | reinterpret_cast<uintptr_t>(R.den)) % 16)
                return ctx;
        } else if (!tiled_prepare(ctx, L, R.vd, R.u, (long long)R.nslots, (long long)L.slot,
                                  R.den)) {
            return ctx;
        }
        ctx.ok = false;
        const size_t n = (size_t)(L.dim == 3 ? L.nz * L.plane : L.nz * L.pitch);
        const bool gz = L.dim == 3 && wants_density_z(L, R.vd);
        // tensor-memory kernel: per-axis tables of the damping mask
        const bool tm = L.dim == 3 && ctx.tm && ctx.tm_tables;
        const size_t ntab = tm ? (size_t)(L.nz + L.nx + L.ny + 32) : 0;
        void* scratch = nullptr;
        SW_CUDA(cudaMallocAsync(&scratch,
                                ((gz ? 3 : 2) * n + ntab) * sizeof(float) + 16 * sizeof(int),
                                st));
        ctx.scratch = scratch;
        float* C = static_cast<float*>(scratch);
        float* Q = C + n;
        float* G = gz ? Q + n : nullptr;
        float* tabs = Q + (gz ? 2 : 1) * n;
        int* words = reinterpret_cast<int*>(tabs + ntab);
        form_coefficients(R.vel, R.damp, C, Q, (long long)n, (float)R.dt, st);
        SW_LAUNCHED("form_coefficients");
        if (G) {
            form_density_z(R.den, G, L, R.W, st);
            SW_LAUNCHED("form_density_z");
            ctx.coefGz = G;
        }
        find_zero_box(Q, L, words, st);
        SW_LAUNCHED("find_zero_box");
        if (tm) {
            damp_face_tables(R.damp, L, words, tabs, tabs + L.nz, tabs + L.nz + L.nx, words + 8,
                             st);
            SW_LAUNCHED("damp_face_tables");
        }
        int box[9];
        SW_CUDA(cudaMemcpyAsync(box, words, sizeof(box), cudaMemcpyDeviceToHost, st));
        SW_CUDA(cudaStreamSynchronize(st));
        bool good = box[6] == 0 && box[1] > box[0] && box[3] > box[2];
        if (L.dim == 3) good = good && box[5] > box[4];
        for (int i = 0; i < 6; i++) ctx.zero_box[i] = good ? box[i] : 0;
        if (tm) {
            ctx.damp = R.damp;
            ctx.damp_tz = tabs;
            ctx.damp_tx = tabs + L.nz;
            ctx.damp_ty = tabs + L.nz + L.nx;
            ctx.damp_faces_ok = good && box[8] == 0;
            ctx.inv_dt = (float)(1.0 / (double)R.dt);
        }
        ctx.coefC = C;
        ctx.coefQ = Q;
        ctx.err = device_words() + 7;
        ctx.ok = true;
    }
    return ctx;
}

// Interior points up to which a 2D float32 run takes the persistent kernel.
constexpr long long kPersistentPoints = 1500000;

// Frees a run's stream-ordered scratch after its last launch.
struct ScratchRelease {
    void* p;
    cudaStream_t st;
    ~ScratchRelease() {
        if (p) cudaFreeAsync(p, st);
    }
};

template <typename T, int DIM, bool VD>
static void run_steps(const Run<T>& R, const Schedule& S, cudaStream_t st,
                      simwave_stats& stats, std::vector<cudaEvent_t>* ev) {
    const Layout& L = R.L;
    const T dt2 = R.dt * R.dt;
    // boundary phases in the reference's order: y, x, z (3D); x, z (2D)
    int phases[3], nphase = 0;
    if (DIM == 3) { phases[0] = 2; phases[1] = 1; phases[2] = 0; nphase = 3; }
    else { phases[0] = 1; phases[1] = 0; nphase = 2; }
    const TiledContext tctx = prepare_tiled<T>(R, st);
    ScratchRelease release{tctx.scratch, st};
    // 2D float32 tiled runs: the step parameters of the owner-computes
    // kernels (sources and boundary edges applied by the tile that holds
    // them, right after its stencil)
    Shot2D shot{};
    bool fused2d = false;
    if constexpr (std::is_same<T, float>::value && DIM == 2) {
        if (tctx.ok)
            fused2d = shot2d_prepare(shot, L, tctx.coefC, tctx.coefQ, R.den, R.vel, R.damp, R.W,
                                     tctx.zero_box, R.src, R.wavelet, R.wavelet_count, R.dt,
                                     R.rec, R.receivers, R.bc) &&
                      shot.fused && !ev;
    }
    if constexpr (std::is_same<T, float>::value && DIM == 2) {
        // small 2D grids: all steps in one persistent launch (the per-step
        // kernels of such grids are bound by their start-up, not their work)
        const size_t nsteps = S.steps.size();
        if (tctx.ok && !ev && !(R.flags & SIMWAVE_FLAG_STEP_LAUNCHES) &&
            L.interior_points() <= kPersistentPoints && nsteps >= 8 && nsteps < (1u << 28)) {
            std::vector<int> tab(3 * nsteps + 2, 0);  // slots per step, 2 barrier words
            for (size_t i = 0; i < nsteps; i++) {
                tab[3 * i] = S.steps[i].next;
                tab[3 * i + 1] = S.steps[i].cur;
                tab[3 * i + 2] = S.steps[i].prev;
            }
            void* dtab = nullptr;
            SW_CUDA(cudaMallocAsync(&dtab, tab.size() * sizeof(int), st));
            ScratchRelease tab_release{dtab, st};
            SW_CUDA(cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(int),
                                    cudaMemcpyHostToDevice, st));
            SW_CUDA(cudaStreamSynchronize(st));  // `tab` is host memory of this call
            for (size_t i = 0; i < nsteps; i++)
                if (R.before_step) R.before_step(i);
            int* itab = static_cast<int*>(dtab);
            if (shot.L.dim == 2 &&
                persistent2d_launch(shot, VD, R.u, itab, (int)nsteps, (long long)R.begin,
                                    reinterpret_cast<unsigned*>(itab + 3 * nsteps), tctx.err,
                                    st)) {
                SW_LAUNCHED("stencil2d_persistent");
                stats.stencil_variant = 2;
                stats.stencil_launches += 1;
                stats.kernel_launches += 1;
                for (size_t i = 0; i < nsteps; i++)
                    if (R.after_step) R.after_step(i);
                return;
            }
        }
    }
    for (size_t i = 0; i < S.steps.size(); i++) {
        const size_t n = R.begin + i;
        T* un = R.u + (size_t)S.steps[i].next * L.slot;
        const T* uc = R.u + (size_t)S.steps[i].cur * L.slot;
        const T* up = R.u + (size_t)S.steps[i].prev * L.slot;
        if (R.before_step) R.before_step(i);
        if constexpr (std::is_same<T, float>::value && DIM == 2) {
            if (fused2d) {  // the whole step in one launch
                step2d_launch(shot, VD, un, uc, up, (long long)n, st);
                SW_LAUNCHED("stencil2d_step");
                stats.stencil_variant = 3;
                stats.stencil_launches++;
                stats.kernel_launches++;
                if (R.after_step) R.after_step(i);
                continue;
            }
        }
        if (ev) SW_CUDA(cudaEventRecord((*ev)[2 * i], st));
        launch_stencil<T, DIM, VD>(R, tctx, un, uc, up, st, &stats.stencil_variant,
                                   &stats.stencil_kernel);
        if (ev) SW_CUDA(cudaEventRecord((*ev)[2 * i + 1], st));
        stats.stencil_launches++;
        stats.kernel_launches++;
        if (R.src.count) {
            inject_sources<T, DIM><<<(unsigned)R.src.count, 128, 0, st>>>(
                un, R.vel, R.damp, L, R.src, R.wavelet, R.wavelet_count, n,
                R.dt, dt2);
            SW_LAUNCHED("inject_sources");
            stats.kernel_launches++;
        }
        for (int ph = 0; ph < nphase; ph++) {
            const int a = phases[ph];
            const int b0 = R.bc[2 * a], b1 = R.bc[2 * a + 1];
            if (b0 == 0 && b1 == 0) continue;
            const int a1 = a == 0 ? 1 : 0;
            const int a2 = DIM == 3 ? (a == 2 ? 1 : 2) : -1;
            const long long lines = (L.extent(a1) - 2 * L.r) *
                                    (a2 >= 0 ? L.extent(a2) - 2 * L.r : 1);
            boundary_phase<T><<<(unsigned)((lines + 255) / 256), 256, 0, st>>>(
                un, L, a, b0, b1);
            SW_LAUNCHED("boundary_phase");
            stats.kernel_launches++;
        }
        if (R.rec.count) {
            const size_t threads = R.rec.count * 32;
            record_receivers<T, DIM><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                R.receivers + (n - 1) * R.rec.count, uc, L, R.rec);
            SW_LAUNCHED("record_receivers");
            stats.kernel_launches++;
        }
        if (R.after_step) R.after_step(i);
    }
}

template <typename T>
static void dispatch_steps(const Run<T>& R, const Schedule& S, cudaStream_t st,
                           simwave_stats& stats, std::vector<cudaEvent_t>* ev) {
    if (R.L.dim == 2 && !R.vd) run_steps<T, 2, false>(R, S, st, stats, ev);
    else if (R.L.dim == 2) run_steps<T, 2, true>(R, S, st, stats, ev);
    else if (!R.vd) run_steps<T, 3, false>(R, S, st, stats, ev);
    else run_steps<T, 3, true>(R, S, st, stats, ev);
}

// Reads and clears the bounded-wait error word (after the stream drained).
static void check_device_words(cudaStream_t st) {
    int* words = device_words();
    int code = 0;
    SW_CUDA(cudaMemcpyAsync(&code, words + 7, sizeof(int), cudaMemcpyDeviceToHost, st));
    SW_CUDA(cudaStreamSynchronize(st));
    if (code) {
        SW_CUDA(cudaMemsetAsync(words + 7, 0, sizeof(int), st));
        SW_CUDA(cudaStreamSynchronize(st));
        fail(code, "a device wait gave up (bounded mbarrier wait expired)");
    }
}

// ---------------------------------------------------------------------------
// validation of sizes and KWS windows (host copies)

static void check_grid(int dim, int order, size_t nz, size_t nx, size_t ny) {
    if (dim != 2 && dim != 3) fail(SIMWAVE_E_ARGUMENT, "dim must be 2 or 3");
    if (order < 2 || order > 20 || order % 2)
        fail(SIMWAVE_E_ARGUMENT, "space_order must be even in 2..20, got " +
                                     std::to_string(order));
    const size_t r = order / 2;
    const size_t ext[3] = {nz, nx, dim == 3 ? ny : 2 * r + 1};
    for (int a = 0; a < 3; a++)
        if (ext[a] < 2 * r + 1)
            fail(SIMWAVE_E_ARGUMENT,
                 "every grid extent must be >= space_order + 1");
    if ((double)nz * nx * (dim == 3 ? ny : 1) > 9.0e15)
        fail(SIMWAVE_E_ARGUMENT, "grid too large");
}

static void check_windows(const char* what, int dim, const size_t* iv,
                          size_t iv_size, const size_t* off,
                          size_t values_size, size_t count,
                          const size_t ext[3]) {
    if (count == 0) return;
    if (!iv || !off) fail(SIMWAVE_E_ARGUMENT, std::string(what) + " arrays missing");
    if (iv_size < count * 2 * dim)
        fail(SIMWAVE_E_ARGUMENT, std::string(what) + "_points_interval too short");
    for (size_t s = 0; s < count; s++) {
        size_t len = 0;
        for (int a = 0; a < dim; a++) {
            const size_t b = iv[s * 2 * dim + 2 * a], e = iv[s * 2 * dim + 2 * a + 1];
            if (b > e || e >= ext[a])
                fail(SIMWAVE_E_ARGUMENT, std::string(what) + " " +
                                             std::to_string(s) +
                                             ": window outside the grid");
            len += e - b + 1;
        }
        if (off[s] > values_size || len > values_size - off[s])
            fail(SIMWAVE_E_ARGUMENT, std::string(what) + " " +
                                         std::to_string(s) +
                                         ": values offset out of range");
    }
}

static void check_time(size_t begin, size_t end, size_t wavelet_size,
                       size_t wavelet_count, size_t nsrc) {
    if (begin < 1) fail(SIMWAVE_E_ARGUMENT, "begin_timestep must be >= 1");
    if (end < begin) return;
    if (nsrc == 0) return;
    const size_t need = wavelet_count > 1 ? end * nsrc : end;
    if (wavelet_size * std::max<size_t>(wavelet_count, 1) < need)
        fail(SIMWAVE_E_ARGUMENT, "wavelet shorter than end_timestep");
}

// ---------------------------------------------------------------------------
// host-pointer entry

template <typename T>
struct HostArgs {
    int dim;
    bool vd;
    T* u;
    const T* vel;
    const T* den;
    const T* damp;
    const T* wavelet;
    size_t wavelet_size, wavelet_count;
    const T* c2;
    const T* c1;
    const size_t* bc;
    const size_t* src_iv;
    size_t src_iv_size;
    const T* src_val;
    size_t src_val_size;
    const size_t* src_off;
    const size_t* rec_iv;
    size_t rec_iv_size;
    const T* rec_val;
    size_t rec_val_size;
    const size_t* rec_off;
    T* receivers;
    size_t nsrc, nrec, nz, nx, ny;
    T dz, dx, dy;
    size_t stride;
    T dt;
    size_t begin, end, order, nslots;
};

// Grid transfers of the host entries: one contiguous copy of the dense host
// array into a dense device staging buffer, then a repack into the pitched
// layout on the device (and the reverse), so that the host link runs at full
// rate; two staging buffers per direction alternate.
// SMs of the current device (cached per device)
static int sm_count() {
    static std::atomic<int> sms[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (!sms[dev & 63]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        sms[dev & 63] = std::max(v, 1);
    }
    return sms[dev & 63];
}

template <typename T>
static void repack(T* dst, const T* src, const Layout& L, bool to_pitched,
                   cudaStream_t st) {
    const long long rows = L.dim == 3 ? L.nz * L.nx : L.nz;
    // small blocks (128 threads, at most 32 registers, no shared memory): one
    // fits beside a block of the time loop's 3D stencil on the same SM, so a
    // snapshot's repack runs while the loop does instead of after it
    repack_rows<T><<<(unsigned)std::min<long long>(rows, 2LL * sm_count()), 128, 0, st>>>(
        dst, src, rows, L.nfast(), L.pitch, L.lead, to_pitched);
    SW_LAUNCHED("repack_rows");
}

// Page-locks caller arrays for the duration of one call (released by the
// destructor); ranges already locked by the caller are used as they are.
// Makes every page of [p, p + bytes) resident, from all host cores, without
// changing its contents (each page has one byte read and written back).
// Freshly allocated arrays (numpy.zeros) are mapped lazily; page-locking them
// would otherwise fault and clear their pages from one thread. The range is
// first advised for transparent huge pages (the contents are unchanged; on
// kernels that grant huge pages only on advice, the snapshot copies into
// large arrays finished sooner: median host call 0.87 s against 1.06 s on
// the 472^3 benchmark shot).
static void fault_in(void* p, size_t bytes) {
    if (!p || bytes < ((size_t)64 << 20)) return;
    const long ps = sysconf(_SC_PAGESIZE);
    const size_t page = ps > 0 ? (size_t)ps : 4096;
    {
        const uintptr_t a = (reinterpret_cast<uintptr_t>(p) + page - 1) / page * page;
        const uintptr_t e = (reinterpret_cast<uintptr_t>(p) + bytes) / page * page;
        if (e > a) madvise(reinterpret_cast<void*>(a), e - a, MADV_HUGEPAGE);
    }
    const unsigned n = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    char* base = static_cast<char*>(p);
    const size_t chunk = (bytes / n + page - 1) / page * page;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < n; t++) {
        const size_t lo = (size_t)t * chunk;
        if (lo >= bytes) break;
        const size_t hi = std::min(bytes, lo + chunk);
        th.emplace_back([=] {
            for (size_t o = lo; o < hi; o += page) {
                volatile char* c = base + o;
                *c = *c;
            }
        });
    }
    for (auto& t : th) t.join();
}

// Whether the halo of one dense host grid (every point with an index within
// r of an edge; with r = 0 the whole grid) is zero bit for bit; the planes
// are scanned from all host cores (3D) or by one thread (2D).
template <typename T>
static bool halo_is_zero(const T* g, int dim, size_t nz, size_t nx, size_t ny, size_t r) {
    using W = typename std::conditional<sizeof(T) == 4, uint32_t, uint64_t>::type;
    const W* w = reinterpret_cast<const W*>(g);
    auto zero = [](const W* p, size_t n) {
        W acc = 0;
        for (size_t i = 0; i < n; i++) acc |= p[i];
        return acc == 0;
    };
    if (dim == 2) {  // rows of nx, z slowest
        for (size_t i = 0; i < nz; i++) {
            const W* row = w + i * nx;
            if (i < r || i >= nz - r || r == 0) {
                if (!zero(row, nx)) return false;
            } else if (!zero(row, r) || !zero(row + nx - r, r)) {
                return false;
            }
        }
        return true;
    }
    auto plane_ok = [&](size_t i) {
        const W* pl = w + i * nx * ny;
        if (i < r || i >= nz - r || r == 0) return zero(pl, nx * ny);
        for (size_t j = 0; j < nx; j++) {
            const W* row = pl + j * ny;
            if (j < r || j >= nx - r) {
                if (!zero(row, ny)) return false;
            } else if (!zero(row, r) || !zero(row + ny - r, r)) {
                return false;
            }
        }
        return true;
    };
    const unsigned n = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<char> ok(n, 1);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < n; t++)
        th.emplace_back([&, t] {
            for (size_t i = t; i < nz && ok[t]; i += n) ok[t] = plane_ok(i);
        });
    for (auto& t : th) t.join();
    for (char c : ok)
        if (!c) return false;
    return true;
}

struct HostPins {
    std::vector<void*> mine;
    cudaError_t last = cudaSuccess;  // the last registration's result
    bool add(const void* p, size_t bytes) {
        if (!p || !bytes) return true;
        fault_in(const_cast<void*>(p), bytes);
        cudaError_t e = cudaHostRegister(const_cast<void*>(p), bytes, cudaHostRegisterDefault);
        last = e;
        if (e == cudaSuccess) {
            mine.push_back(const_cast<void*>(p));
            return true;
        }
        cudaGetLastError();  // clear
        return e == cudaErrorHostMemoryAlreadyRegistered;
    }
    void release() {
        for (void* p : mine) cudaHostUnregister(p);
        mine.clear();
    }
    ~HostPins() { release(); }
};

template <typename T>
static void* upload(Buffer& b, const void* src, size_t bytes, cudaStream_t st,
                    size_t* counted) {
    void* p = b.ensure(std::max<size_t>(bytes, 16));
    if (bytes) SW_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, st));
    *counted += bytes;
    return p;
}

template <typename T>
static double host_forward(const HostArgs<T>& A) {
    const auto t0 = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lock(g_mutex);
    simwave_stats stats;
    std::memset(&stats, 0, sizeof(stats));

    check_grid(A.dim, (int)A.order, A.nz, A.nx, A.ny);
    const size_t ext[3] = {A.nz, A.nx, A.dim == 3 ? A.ny : 1};
    if (!A.u || !A.vel || !A.damp || (A.vd && (!A.den || !A.c1)) || !A.c2 ||
        !A.bc || (A.nrec && !A.receivers) || (A.nsrc && !A.wavelet))
        fail(SIMWAVE_E_ARGUMENT, "null array argument");
    for (int e = 0; e < 2 * A.dim; e++)
        if (A.bc[e] > 2) fail(SIMWAVE_E_ARGUMENT, "boundary code must be 0, 1 or 2");
    check_windows("src", A.dim, A.src_iv, A.src_iv_size, A.src_off,
                  A.src_val_size, A.nsrc, ext);
    check_windows("rec", A.dim, A.rec_iv, A.rec_iv_size, A.rec_off,
                  A.rec_val_size, A.nrec, ext);
    check_time(A.begin, A.end, A.wavelet_size, A.wavelet_count, A.nsrc);
    Schedule S = make_schedule(A.begin, A.end, A.stride, A.nslots);

    Layout L;
    L.dim = A.dim;
    L.r = (int)(A.order / 2);
    L.nz = (long long)A.nz;
    L.nx = (long long)A.nx;
    L.ny = A.dim == 3 ? (long long)A.ny : 1;
    size_t pitch, lead;
    choose_layout((size_t)L.nfast(), L.r, (int)sizeof(T), &pitch, &lead);
    L.pitch = (long long)pitch;
    L.lead = (long long)lead;
    L.plane = A.dim == 3 ? L.nx * L.pitch : L.pitch;
    L.slot = A.dim == 3 ? L.nz * L.plane : L.nz * L.pitch;

    Arena& ar = arena_for_current_device();
    cudaStream_t st = ar.stream;
    const size_t slot_bytes = (size_t)L.slot * sizeof(T);
    T* du = (T*)ar.u.ensure(slot_bytes * A.nslots);
    T* dvel = (T*)ar.vel.ensure(slot_bytes);
    T* dden = A.vd ? (T*)ar.den.ensure(slot_bytes) : nullptr;
    T* ddamp = (T*)ar.damp.ensure(slot_bytes);
    const size_t rec_rows = A.end >= A.begin ? A.end - A.begin + 1 : 0;
    T* drec = (T*)ar.rec.ensure(std::max<size_t>(A.end * A.nrec * sizeof(T), 16));

    size_t h2d = 0, d2h = 0;
    const size_t dense = (size_t)(L.nz * L.nx * L.ny);
    const size_t dense_bytes = dense * sizeof(T);
    cudaStream_t cin = ar.copy_in, cout = ar.copy_out;
    // events: [0,2) staging-in free, [2,4) staging-out free, [4] fields
    // ready, [5, 5 + nslots) slot ready, [5 + nslots, 5 + 2 nslots) slot done
    const size_t EV_IN = 0, EV_OUT = 2, EV_FIELDS = 4, EV_READY = 5;
    const size_t EV_DONE = EV_READY + A.nslots;
    ar.event(EV_DONE + A.nslots);
    SW_CUDA(cudaEventRecord(ar.event(EV_IN), cin));
    SW_CUDA(cudaEventRecord(ar.event(EV_IN + 1), cin));
    SW_CUDA(cudaEventRecord(ar.event(EV_OUT), cout));
    SW_CUDA(cudaEventRecord(ar.event(EV_OUT + 1), cout));
    int in_turn = 0, out_turn = 0;
    // transfer mode: AUTO page-locks the caller's grids for the call; AUTO
    // and STAGED move each grid as one contiguous copy through a dense
    // device staging buffer plus a repack kernel (pitched <-> dense); DIRECT
    // (coherent host links, pageable arrays) lets the repack kernel read and
    // write the host arrays itself, with no staging
    // SIMWAVE_TRACE set: phase times of this call on stderr
    const bool trace = std::getenv("SIMWAVE_TRACE") != nullptr;
    auto stamp = [&](const char* what) {
        if (trace)
            std::fprintf(stderr, "simwave host entry: %-14s %9.3f ms\n", what,
                         1e3 * std::chrono::duration<double>(
                                   std::chrono::steady_clock::now() - t0).count());
    };
    stamp("checked");
    HostPins pins;
    bool pinned = false;
    if (g_transfer_mode == SIMWAVE_TRANSFER_AUTO) {
        pinned = pins.add(A.u, dense_bytes * A.nslots) && pins.add(A.vel, dense_bytes) &&
                 pins.add(A.damp, dense_bytes) && (!A.vd || pins.add(A.den, dense_bytes));
        if (!pinned) pins.release();
        // the record's rows too: a pageable copy of a freshly allocated
        // record faulted its pages in after the time loop
        if (pinned && rec_rows && A.nrec && A.receivers)
            pins.add(A.receivers + (A.begin - 1) * A.nrec, rec_rows * A.nrec * sizeof(T));
    }
    if (trace && !pinned)
        std::fprintf(stderr, "simwave host entry: page-locking failed: %s\n",
                     cudaGetErrorString(pins.last));
    stamp(pinned ? "pinned" : "not pinned");
    const bool direct = !pinned && ar.host_access && g_transfer_mode == SIMWAVE_TRANSFER_DIRECT;
    T* sin[2] = {nullptr, nullptr};
    T* sout[2] = {nullptr, nullptr};
    if (!direct)
        for (int b = 0; b < 2; b++) {
            sin[b] = (T*)ar.stage_in[b].ensure(dense_bytes);
            sout[b] = (T*)ar.stage_out[b].ensure(dense_bytes);
        }
    // uploads (also from page-locked arrays): one contiguous copy into a
    // dense device buffer, then a repack into the pitched layout; pitched
    // copies move one short row per descriptor (about 20 GB/s here against
    // about 200 GB/s for one contiguous copy)
    auto upload_grid = [&](T* dst, const T* src) {
        h2d += dense_bytes;
        if (direct) {
            repack<T>(dst, src, L, true, cin);
            return;
        }
        const int b = in_turn++ & 1;
        SW_CUDA(cudaStreamWaitEvent(cin, ar.event(EV_IN + b), 0));
        SW_CUDA(cudaMemcpyAsync(sin[b], src, dense_bytes, cudaMemcpyHostToDevice, cin));
        repack<T>(dst, sin[b], L, true, cin);
        SW_CUDA(cudaEventRecord(ar.event(EV_IN + b), cin));
    };
    // downloads (also to page-locked arrays): a repack into a dense device
    // buffer, then one contiguous copy; pitched copies of short rows (one
    // per x row of a grid) left the host link running at a fraction of its
    // rate, so snapshots finished up to 0.6 s after the time loop
    auto download_grid = [&](T* dst, const T* src) {
        d2h += dense_bytes;
        if (direct) {
            repack<T>(dst, src, L, false, cout);
            return;
        }
        const int b = out_turn++ & 1;
        SW_CUDA(cudaStreamWaitEvent(cout, ar.event(EV_OUT + b), 0));
        repack<T>(sout[b], src, L, false, cout);
        SW_CUDA(cudaMemcpyAsync(dst, sout[b], dense_bytes, cudaMemcpyDeviceToHost, cout));
        SW_CUDA(cudaEventRecord(ar.event(EV_OUT + b), cout));
    };
    // with the trace: device time from the call's first upload to the first
    // step and across the time loop
    cudaEvent_t tr_ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (trace) {
        for (auto& e : tr_ev) SW_CUDA(cudaEventCreate(&e));
        SW_CUDA(cudaEventRecord(tr_ev[0], cin));
    }
    // models and KWS tables first, then the slots in the order the steps
    // first touch them
    upload_grid(dvel, A.vel);
    if (A.vd) upload_grid(dden, A.den);
    upload_grid(ddamp, A.damp);
    const size_t wlen = A.wavelet_size * std::max<size_t>(A.wavelet_count, 1);
    T* dw = (T*)upload<T>(ar.wavelet, A.wavelet, A.nsrc ? wlen * sizeof(T) : 0, cin, &h2d);
    size_t* dsiv = (size_t*)upload<T>(ar.src_iv, A.src_iv, A.nsrc * 2 * A.dim * sizeof(size_t), cin, &h2d);
    T* dsval = (T*)upload<T>(ar.src_val, A.src_val, A.nsrc ? A.src_val_size * sizeof(T) : 0, cin, &h2d);
    size_t* dsoff = (size_t*)upload<T>(ar.src_off, A.src_off, A.nsrc ? A.nsrc * sizeof(size_t) : 0, cin, &h2d);
    size_t* driv = (size_t*)upload<T>(ar.rec_iv, A.rec_iv, A.nrec * 2 * A.dim * sizeof(size_t), cin, &h2d);
    T* drval = (T*)upload<T>(ar.rec_val, A.rec_val, A.nrec ? A.rec_val_size * sizeof(T) : 0, cin, &h2d);
    size_t* droff = (size_t*)upload<T>(ar.rec_off, A.rec_off, A.nrec ? A.nrec * sizeof(size_t) : 0, cin, &h2d);
    SW_CUDA(cudaEventRecord(ar.event(EV_FIELDS), cin));
    // physical slot p starts with host slot p; upload those the run reads or
    // returns, in first-use order
    std::vector<size_t> first_use(A.nslots, (size_t)-1), last_write(A.nslots, (size_t)-1);
    std::vector<size_t> first_read(A.nslots, (size_t)-1), first_write(A.nslots, (size_t)-1);
    for (size_t i = 0; i < S.steps.size(); i++) {
        const int ps[3] = {S.steps[i].prev, S.steps[i].cur, S.steps[i].next};
        for (int q = 0; q < 3; q++)
            if (first_use[ps[q]] == (size_t)-1) first_use[ps[q]] = i;
        for (int q = 0; q < 2; q++)
            if (first_read[ps[q]] == (size_t)-1) first_read[ps[q]] = i;
        if (first_write[ps[2]] == (size_t)-1) first_write[ps[2]] = i;
        last_write[S.steps[i].next] = i;
    }
    std::vector<int> inv(A.nslots);
    for (size_t j = 0; j < A.nslots; j++) inv[S.perm[j]] = (int)j;
    std::vector<char> needed(A.nslots, 0), uploaded(A.nslots, 0);
    for (size_t p = 0; p < A.nslots; p++)
        needed[p] = first_use[p] != (size_t)-1 || inv[p] != (int)p;
    std::vector<size_t> order;
    for (size_t p = 0; p < A.nslots; p++)
        if (needed[p]) order.push_back(p);
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return first_use[a] < first_use[b]; });
    // a slot the steps write before they read it keeps only its halo from
    // the host (every interior point is overwritten first); when that halo
    // is zero bit for bit (Solver.forward's zero-filled u_full), the slot is
    // cleared on the device instead of uploaded
    // (a slot read first is cleared the same way when it is zero throughout)
    for (size_t p : order) {
        const bool written_first = first_write[p] != (size_t)-1 && first_write[p] < first_read[p];
        if (halo_is_zero<T>(A.u + p * dense, A.dim, A.nz, A.nx, A.dim == 3 ? A.ny : 1,
                            written_first ? (size_t)L.r : 0)) {
            SW_CUDA(cudaMemsetAsync(du + p * L.slot, 0, (size_t)L.slot * sizeof(T), cin));
        } else {
            upload_grid(du + p * L.slot, A.u + p * dense);
        }
        SW_CUDA(cudaEventRecord(ar.event(EV_READY + p), cin));
        uploaded[p] = 1;
    }
    // the time loop waits for the models, and for each slot before its
    // first use; a slot's result leaves as soon as its last write is queued
    SW_CUDA(cudaStreamWaitEvent(st, ar.event(EV_FIELDS), 0));
    std::vector<std::vector<int>> start_at(S.steps.size() + 1), done_at(S.steps.size() + 1);
    for (size_t p = 0; p < A.nslots; p++) {
        if (first_use[p] != (size_t)-1) start_at[first_use[p]].push_back((int)p);
        if (last_write[p] != (size_t)-1) done_at[last_write[p]].push_back((int)p);
    }
    auto emit = [&](int p) {  // result of physical slot p -> host slot inv[p]
        SW_CUDA(cudaEventRecord(ar.event(EV_DONE + p), st));
        SW_CUDA(cudaStreamWaitEvent(cout, ar.event(EV_DONE + p), 0));
        download_grid(A.u + (size_t)inv[p] * dense, du + (size_t)p * L.slot);
    };
    Run<T> R;
    R.L = L;
    R.vd = A.vd;
    R.u = du;
    R.nslots = A.nslots;
    R.vel = dvel;
    R.den = dden;
    R.damp = ddamp;
    R.wavelet = dw;
    R.wavelet_count = A.wavelet_count;
    R.W = make_weights<T>(A.c2, A.vd ? A.c1 : nullptr, L.r, (double)A.dz,
                          (double)A.dx, A.dim == 3 ? (double)A.dy : 1.0);
    for (int e = 0; e < 6; e++) R.bc[e] = e < 2 * A.dim ? (int)A.bc[e] : 0;
    R.src = Windows<T>{dsiv, dsval, dsoff, A.nsrc};
    R.rec = Windows<T>{driv, drval, droff, A.nrec};
    R.receivers = drec;
    R.begin = A.begin;
    R.end = A.end;
    R.stride = A.stride;
    R.dt = A.dt;
    R.flags = 0;
    R.before_step = [&](size_t i) {
        for (int p : start_at[i]) SW_CUDA(cudaStreamWaitEvent(st, ar.event(EV_READY + p), 0));
    };
    // a slot's final content is known once the step after its last write has
    // been queued (that step may still read it, which does not change it)
    R.after_step = [&](size_t i) {
        for (int p : done_at[i]) emit(p);
    };
    stamp("uploads queued");
    if (trace) SW_CUDA(cudaEventRecord(tr_ev[1], st));
    dispatch_steps<T>(R, S, st, stats, nullptr);
    if (trace) SW_CUDA(cudaEventRecord(tr_ev[2], st));
    stamp("steps queued");

    // slots that changed identity without being written
    for (size_t p = 0; p < A.nslots; p++)
        if (last_write[p] == (size_t)-1 && inv[p] != (int)p) {
            SW_CUDA(cudaStreamWaitEvent(st, ar.event(EV_READY + p), 0));
            emit((int)p);
        }
    if (rec_rows && A.nrec) {
        const size_t off = (A.begin - 1) * A.nrec;
        SW_CUDA(cudaMemcpyAsync(A.receivers + off, drec + off,
                                rec_rows * A.nrec * sizeof(T),
                                cudaMemcpyDeviceToHost, st));
        d2h += rec_rows * A.nrec * sizeof(T);
    }
    if (trace) {
        SW_CUDA(cudaEventRecord(tr_ev[3], st));
        SW_CUDA(cudaEventRecord(tr_ev[4], cout));
        SW_CUDA(cudaEventRecord(tr_ev[5], cin));
    }
    SW_CUDA(cudaStreamSynchronize(st));
    SW_CUDA(cudaStreamSynchronize(cin));
    SW_CUDA(cudaStreamSynchronize(cout));
    stamp("all done");
    if (trace) {
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, tr_ev[0], tr_ev[1]);
        cudaEventElapsedTime(&b, tr_ev[1], tr_ev[2]);
        std::fprintf(stderr, "simwave host entry: device: uploads start -> loop start %.3f ms, "
                             "time loop %.3f ms\n", a, b);
        float c = 0.f, d = 0.f, e = 0.f;
        cudaEventElapsedTime(&c, tr_ev[0], tr_ev[3]);
        cudaEventElapsedTime(&d, tr_ev[0], tr_ev[4]);
        cudaEventElapsedTime(&e, tr_ev[0], tr_ev[5]);
        std::fprintf(stderr, "simwave host entry: device: from uploads start, loop stream done "
                             "%.3f ms, copies out done %.3f ms, copies in done %.3f ms\n", c, d, e);
        for (auto& e : tr_ev) cudaEventDestroy(e);
    }
    pins.release();
    stamp("unpinned");
    check_device_words(st);
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stats.seconds = secs;
    stats.updates = (double)L.interior_points() * (double)S.steps.size();
    stats.h2d_bytes = h2d;
    stats.d2h_bytes = d2h;
    g_last_stats = stats;
    return secs;
}

template <typename T>
static double host_entry(const HostArgs<T>& A) {
    try {
        g_last_error.clear();
        return host_forward<T>(A);
    } catch (const Failure& f) {
        g_last_error = f.message;
        return -(double)f.code;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return -(double)SIMWAVE_E_ARGUMENT;
    }
}

// ---------------------------------------------------------------------------
// device-pointer entry

template <typename T>
static int device_forward(const simwave_problem* P, cudaStream_t st) {
    const auto t0 = std::chrono::steady_clock::now();
    simwave_stats stats;
    std::memset(&stats, 0, sizeof(stats));
    if (!P) fail(SIMWAVE_E_ARGUMENT, "null problem");
    check_grid(P->dim, P->space_order, P->nz, P->nx, P->ny);
    const bool vd = P->variable_density != 0;
    const size_t ext[3] = {P->nz, P->nx, P->dim == 3 ? P->ny : 1};
    if (!P->u || !P->velocity || !P->damp || (vd && (!P->density || !P->coeff_order1)) ||
        !P->coeff_order2 || !P->boundary_conditions ||
        (P->num_receivers && !P->receivers) || (P->num_sources && !P->wavelet))
        fail(SIMWAVE_E_ARGUMENT, "null array argument");
    for (int e = 0; e < 2 * P->dim; e++)
        if (P->boundary_conditions[e] > 2)
            fail(SIMWAVE_E_ARGUMENT, "boundary code must be 0, 1 or 2");
    const size_t nfast = P->dim == 3 ? P->ny : P->nx;
    if (P->pitch < P->lead + nfast) fail(SIMWAVE_E_ARGUMENT, "pitch < lead + fastest extent");
    const size_t grid_elems = P->dim == 3 ? P->nz * P->nx * P->pitch : P->nz * P->pitch;
    if (P->num_snapshots > 1 && P->slot_stride < grid_elems)
        fail(SIMWAVE_E_ARGUMENT, "slot_stride smaller than one grid");
    check_time(P->begin_timestep, P->end_timestep, P->wavelet_size,
               P->wavelet_count, P->num_sources);
    if (!(P->flags & SIMWAVE_FLAG_WINDOWS_CHECKED)) {
        // copy the windows to the host and check them
        for (int which = 0; which < 2; which++) {
            const size_t count = which ? P->num_receivers : P->num_sources;
            if (!count) continue;
            const size_t* div = which ? P->rec_points_interval : P->src_points_interval;
            const size_t* doff = which ? P->rec_points_values_offset : P->src_points_values_offset;
            std::vector<size_t> iv(count * 2 * P->dim), off(count);
            SW_CUDA(cudaMemcpyAsync(iv.data(), div, iv.size() * sizeof(size_t),
                                    cudaMemcpyDeviceToHost, st));
            SW_CUDA(cudaMemcpyAsync(off.data(), doff, off.size() * sizeof(size_t),
                                    cudaMemcpyDeviceToHost, st));
            SW_CUDA(cudaStreamSynchronize(st));
            check_windows(which ? "rec" : "src", P->dim, iv.data(), iv.size(),
                          off.data(),
                          which ? P->rec_points_values_size : P->src_points_values_size,
                          count, ext);
        }
    }
    Schedule S = make_schedule(P->begin_timestep, P->end_timestep,
                               P->saving_stride, P->num_snapshots);
    Layout L;
    L.dim = P->dim;
    L.r = P->space_order / 2;
    L.nz = (long long)P->nz;
    L.nx = (long long)P->nx;
    L.ny = P->dim == 3 ? (long long)P->ny : 1;
    L.pitch = (long long)P->pitch;
    L.lead = (long long)P->lead;
    L.plane = P->dim == 3 ? L.nx * L.pitch : L.pitch;
    L.slot = (long long)P->slot_stride;

    Run<T> R;
    R.L = L;
    R.vd = vd;
    R.u = (T*)P->u;
    R.nslots = P->num_snapshots;
    R.vel = (const T*)P->velocity;
    R.den = (const T*)P->density;
    R.damp = (const T*)P->damp;
    R.wavelet = (const T*)P->wavelet;
    R.wavelet_count = P->wavelet_count;
    R.W = make_weights<T>((const T*)P->coeff_order2,
                          vd ? (const T*)P->coeff_order1 : nullptr, L.r, P->dz,
                          P->dx, P->dim == 3 ? P->dy : 1.0);
    for (int e = 0; e < 6; e++)
        R.bc[e] = e < 2 * P->dim ? (int)P->boundary_conditions[e] : 0;
    R.src = Windows<T>{P->src_points_interval, (const T*)P->src_points_values,
                       P->src_points_values_offset, P->num_sources};
    R.rec = Windows<T>{P->rec_points_interval, (const T*)P->rec_points_values,
                       P->rec_points_values_offset, P->num_receivers};
    R.receivers = (T*)P->receivers;
    R.begin = P->begin_timestep;
    R.end = P->end_timestep;
    R.stride = P->saving_stride;
    R.dt = (T)P->dt;
    R.flags = P->flags;

    std::vector<cudaEvent_t>* ev = nullptr;
    std::vector<cudaEvent_t> events;
    if (P->flags & SIMWAVE_FLAG_TIME_KERNELS) {
        int dev = 0;
        SW_CUDA(cudaGetDevice(&dev));
        std::lock_guard<std::mutex> lock(g_event_mutex);
        auto& pool = g_event_pool[dev];
        while (pool.size() < 2 * S.steps.size()) {
            cudaEvent_t e;
            SW_CUDA(cudaEventCreate(&e));
            pool.push_back(e);
        }
        events.assign(pool.begin(), pool.begin() + 2 * S.steps.size());
        ev = &events;
    }
    dispatch_steps<T>(R, S, st, stats, ev);

    // restore the logical slot order where the even-stride exchanges moved it
    bool moved = false;
    for (size_t j = 0; j < P->num_snapshots; j++) moved |= S.perm[j] != (int)j;
    if (moved) {
        const size_t bytes = grid_elems * sizeof(T);
        void* tmpv = nullptr;
        SW_CUDA(cudaMallocAsync(&tmpv, bytes, st));
        ScratchRelease tmp_release{tmpv, st};
        T* tmp = static_cast<T*>(tmpv);
        std::vector<char> done(P->num_snapshots, 0);
        T* base = (T*)P->u;
        for (size_t j = 0; j < P->num_snapshots; j++) {
            if (done[j] || S.perm[j] == (int)j) continue;
            // cycle j <- perm[j] <- perm[perm[j]] ...
            SW_CUDA(cudaMemcpyAsync(tmp, base + j * L.slot, bytes, cudaMemcpyDeviceToDevice, st));
            size_t cur = j;
            while (true) {
                const size_t src = (size_t)S.perm[cur];
                done[cur] = 1;
                if (src == j) {
                    SW_CUDA(cudaMemcpyAsync(base + cur * L.slot, tmp, bytes, cudaMemcpyDeviceToDevice, st));
                    break;
                }
                SW_CUDA(cudaMemcpyAsync(base + cur * L.slot, base + src * L.slot, bytes,
                                        cudaMemcpyDeviceToDevice, st));
                cur = src;
            }
        }
    }
    if (ev) {
        SW_CUDA(cudaStreamSynchronize(st));
        check_device_words(st);
        double ms = 0;
        for (size_t i = 0; i < S.steps.size(); i++) {
            float t = 0;
            SW_CUDA(cudaEventElapsedTime(&t, events[2 * i], events[2 * i + 1]));
            ms += t;
        }
        stats.stencil_ms = ms;
    }
    stats.seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stats.updates = (double)L.interior_points() * (double)S.steps.size();
    g_last_stats = stats;
    return SIMWAVE_OK;
}

}  // namespace sw

// ---------------------------------------------------------------------------
// C ABI

using sw::HostArgs;

#define SW_HOST_ARGS_COMMON(T)                                                \
    A.wavelet = wavelet; A.wavelet_size = wavelet_size;                       \
    A.wavelet_count = wavelet_count; A.bc = boundary_conditions;              \
    A.src_iv = src_points_interval; A.src_iv_size = src_points_interval_size; \
    A.src_val = src_points_values; A.src_val_size = src_points_values_size;   \
    A.src_off = src_points_values_offset; A.rec_iv = rec_points_interval;     \
    A.rec_iv_size = rec_points_interval_size; A.rec_val = rec_points_values;  \
    A.rec_val_size = rec_points_values_size;                                  \
    A.rec_off = rec_points_values_offset; A.receivers = receivers;            \
    A.nsrc = num_sources; A.nrec = num_receivers; A.stride = saving_stride;   \
    A.dt = dt; A.begin = begin_timestep; A.end = end_timestep;                \
    A.order = space_order; A.nslots = num_snapshots; A.u = u;                 \
    A.vel = velocity; A.damp = damp;

#define SW_DEFINE_2D_CD(SFX, T)                                               \
    extern "C" double simwave_forward_2d_cd_##SFX(                            \
        T* u, T* velocity, T* damp, T* wavelet, size_t wavelet_size,          \
        size_t wavelet_count, T* coeff, size_t* boundary_conditions,          \
        size_t* src_points_interval, size_t src_points_interval_size,         \
        T* src_points_values, size_t src_points_values_size,                  \
        size_t* src_points_values_offset, size_t* rec_points_interval,        \
        size_t rec_points_interval_size, T* rec_points_values,                \
        size_t rec_points_values_size, size_t* rec_points_values_offset,      \
        T* receivers, size_t num_sources, size_t num_receivers, size_t nz,    \
        size_t nx, T dz, T dx, size_t saving_stride, T dt,                    \
        size_t begin_timestep, size_t end_timestep, size_t space_order,       \
        size_t num_snapshots) {                                               \
        HostArgs<T> A{};                                                      \
        SW_HOST_ARGS_COMMON(T)                                                \
        A.dim = 2; A.vd = false; A.den = nullptr; A.c2 = coeff;               \
        A.c1 = nullptr; A.nz = nz; A.nx = nx; A.ny = 1; A.dz = dz;            \
        A.dx = dx; A.dy = 1;                                                  \
        return sw::host_entry<T>(A);                                          \
    }

#define SW_DEFINE_2D_VD(SFX, T)                                               \
    extern "C" double simwave_forward_2d_vd_##SFX(                            \
        T* u, T* velocity, T* density, T* damp, T* wavelet,                   \
        size_t wavelet_size, size_t wavelet_count, T* coeff_order2,           \
        T* coeff_order1, size_t* boundary_conditions,                         \
        size_t* src_points_interval, size_t src_points_interval_size,         \
        T* src_points_values, size_t src_points_values_size,                  \
        size_t* src_points_values_offset, size_t* rec_points_interval,        \
        size_t rec_points_interval_size, T* rec_points_values,                \
        size_t rec_points_values_size, size_t* rec_points_values_offset,      \
        T* receivers, size_t num_sources, size_t num_receivers, size_t nz,    \
        size_t nx, T dz, T dx, size_t saving_stride, T dt,                    \
        size_t begin_timestep, size_t end_timestep, size_t space_order,       \
        size_t num_snapshots) {                                               \
        HostArgs<T> A{};                                                      \
        SW_HOST_ARGS_COMMON(T)                                                \
        A.dim = 2; A.vd = true; A.den = density; A.c2 = coeff_order2;         \
        A.c1 = coeff_order1; A.nz = nz; A.nx = nx; A.ny = 1; A.dz = dz;       \
        A.dx = dx; A.dy = 1;                                                  \
        return sw::host_entry<T>(A);                                          \
    }

#define SW_DEFINE_3D_CD(SFX, T)                                               \
    extern "C" double simwave_forward_3d_cd_##SFX(                            \
        T* u, T* velocity, T* damp, T* wavelet, size_t wavelet_size,          \
        size_t wavelet_count, T* coeff, size_t* boundary_conditions,          \
        size_t* src_points_interval, size_t src_points_interval_size,         \
        T* src_points_values, size_t src_points_values_size,                  \
        size_t* src_points_values_offset, size_t* rec_points_interval,        \
        size_t rec_points_interval_size, T* rec_points_values,                \
        size_t rec_points_values_size, size_t* rec_points_values_offset,      \
        T* receivers, size_t num_sources, size_t num_receivers, size_t nz,    \
        size_t nx, size_t ny, T dz, T dx, T dy, size_t saving_stride, T dt,   \
        size_t begin_timestep, size_t end_timestep, size_t space_order,       \
        size_t num_snapshots) {                                               \
        HostArgs<T> A{};                                                      \
        SW_HOST_ARGS_COMMON(T)                                                \
        A.dim = 3; A.vd = false; A.den = nullptr; A.c2 = coeff;               \
        A.c1 = nullptr; A.nz = nz; A.nx = nx; A.ny = ny; A.dz = dz;           \
        A.dx = dx; A.dy = dy;                                                 \
        return sw::host_entry<T>(A);                                          \
    }

#define SW_DEFINE_3D_VD(SFX, T)                                               \
    extern "C" double simwave_forward_3d_vd_##SFX(                            \
        T* u, T* velocity, T* density, T* damp, T* wavelet,                   \
        size_t wavelet_size, size_t wavelet_count, T* coeff_order2,           \
        T* coeff_order1, size_t* boundary_conditions,                         \
        size_t* src_points_interval, size_t src_points_interval_size,         \
        T* src_points_values, size_t src_points_values_size,                  \
        size_t* src_points_values_offset, size_t* rec_points_interval,        \
        size_t rec_points_interval_size, T* rec_points_values,                \
        size_t rec_points_values_size, size_t* rec_points_values_offset,      \
        T* receivers, size_t num_sources, size_t num_receivers, size_t nz,    \
        size_t nx, size_t ny, T dz, T dx, T dy, size_t saving_stride, T dt,   \
        size_t begin_timestep, size_t end_timestep, size_t space_order,       \
        size_t num_snapshots) {                                               \
        HostArgs<T> A{};                                                      \
        SW_HOST_ARGS_COMMON(T)                                                \
        A.dim = 3; A.vd = true; A.den = density; A.c2 = coeff_order2;         \
        A.c1 = coeff_order1; A.nz = nz; A.nx = nx; A.ny = ny; A.dz = dz;      \
        A.dx = dx; A.dy = dy;                                                 \
        return sw::host_entry<T>(A);                                          \
    }

SW_DEFINE_2D_CD(f32, float)
SW_DEFINE_2D_CD(f64, double)
SW_DEFINE_2D_VD(f32, float)
SW_DEFINE_2D_VD(f64, double)
SW_DEFINE_3D_CD(f32, float)
SW_DEFINE_3D_CD(f64, double)
SW_DEFINE_3D_VD(f32, float)
SW_DEFINE_3D_VD(f64, double)

extern "C" const char* simwave_last_error(void) { return sw::g_last_error.c_str(); }

extern "C" int simwave_forward_device(const simwave_problem* problem, void* stream) {
    try {
        sw::g_last_error.clear();
        if (!problem) sw::fail(SIMWAVE_E_ARGUMENT, "null problem");
        if (problem->precision == 4)
            return sw::device_forward<float>(problem, (cudaStream_t)stream);
        if (problem->precision == 8)
            return sw::device_forward<double>(problem, (cudaStream_t)stream);
        sw::fail(SIMWAVE_E_ARGUMENT, "precision must be 4 or 8");
    } catch (const sw::Failure& f) {
        sw::g_last_error = f.message;
        return f.code;
    } catch (const std::exception& e) {
        sw::g_last_error = e.what();
        return SIMWAVE_E_ARGUMENT;
    }
}

extern "C" int simwave_device_status(void* stream) {
    try {
        sw::g_last_error.clear();
        SW_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
        sw::check_device_words((cudaStream_t)stream);
        return SIMWAVE_OK;
    } catch (const sw::Failure& f) {
        sw::g_last_error = f.message;
        return f.code;
    }
}

extern "C" int simwave_set_kernel_policy(int policy) {
    if (policy < SIMWAVE_POLICY_AUTO || policy > SIMWAVE_POLICY_STAGE_RELEASE)
        return SIMWAVE_E_ARGUMENT;
    sw::set_kernel_policy(policy);
    return SIMWAVE_OK;
}

extern "C" int simwave_set_transfer_mode(int mode) {
    if (mode < SIMWAVE_TRANSFER_AUTO || mode > SIMWAVE_TRANSFER_DIRECT) return SIMWAVE_E_ARGUMENT;
    std::lock_guard<std::mutex> lock(sw::g_mutex);
    sw::g_transfer_mode = mode;
    return SIMWAVE_OK;
}

extern "C" int simwave_last_stats(simwave_stats* out) {
    if (!out) return SIMWAVE_E_ARGUMENT;
    *out = sw::g_last_stats;
    return SIMWAVE_OK;
}

extern "C" int simwave_layout(size_t fastest_extent, int space_order,
                              int precision, size_t* pitch, size_t* lead) {
    if (!pitch || !lead || (precision != 4 && precision != 8) ||
        space_order < 2 || space_order > 20 || space_order % 2)
        return SIMWAVE_E_ARGUMENT;
    sw::choose_layout(fastest_extent, space_order / 2, precision, pitch, lead);
    return SIMWAVE_OK;
}
