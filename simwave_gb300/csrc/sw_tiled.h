// sw_tiled.h -- tiled 3D float32 stencil (sw_stencil_tiled.cu).
#pragma once

#include "sw_common.cuh"

namespace sw {

// Per-run state of the tiled kernel: TMA descriptors of the wavefield slots
// and of the density, the box where the damping mask is zero, and the device
// error word that bounded waits set on expiry.
struct TiledContext {
    bool ok = false;
    alignas(64) unsigned char map_u[128];      // boxes of the scalar kernel
    alignas(64) unsigned char map_rho[128];
    alignas(64) unsigned char map_u_vec[128];  // boxes of the float4 kernel
    alignas(64) unsigned char map_rho_vec[128];
    bool vec = false;                          // float4 kernel usable
    const float* u_base = nullptr;
    long long slot_stride = 0;
    int zero_box[6] = {0, 0, 0, 0, 0, 0};  // z0, z1, x0, x1, y0, y1 (empty)
    int* err = nullptr;
    const float* coefC = nullptr;  // per-point coefficients (same layout as u)
    const float* coefQ = nullptr;
    const float* coefGz = nullptr; // density z term (variable density), or null
    void* scratch = nullptr;       // the run's coefficient/zero-box scratch
    // kernels of sw_stencil_tmem.cu (TMEM and stage-release policies)
    alignas(64) unsigned char map_u_tm[128];   // boxes of tm_rows x rows
    alignas(64) unsigned char map_rho_tm[128];
    bool tm = false;               // descriptors encoded
    int tm_rows = 8;               // x rows per CTA (8 or 12)
    bool tm_tables = false;        // the kernel reads the per-axis damping tables
    const float* damp = nullptr;   // the damping mask (pitched like u)
    const float* damp_tz = nullptr;  // mask along the zero box's centre lines
    const float* damp_tx = nullptr;
    const float* damp_ty = nullptr;
    int damp_faces_ok = 0;         // tables match every one-axis-outside point
    float inv_dt = 0.f;
};

// Encodes the descriptors; false when the layout or alignment does not suit
// the tiled kernel (the generic kernel then runs).
bool tiled_prepare(TiledContext& ctx, const Layout& L, bool vd, float* u_base,
                   long long nslots, long long slot_stride, const float* den);

// `coefC` and `coefQ` are the per-point coefficients of form_coefficients.
// Returns the SIMWAVE_POLICY_* of the kernel launched.
int tiled_launch(const TiledContext& ctx, bool vd, float* un, const float* uc,
                  const float* up, const float* coefC, const float* den,
                  const float* coefQ, const Layout& L, const Weights<float>& W,
                  float dt, float dt2, cudaStream_t st);

// C = (dt^2 v^2) / (1 + Q), Q = damp dt v^2 / 2, elementwise over n values,
// with the reference's operation order (all IEEE round-to-nearest).
void form_coefficients(const float* vel, const float* damp, float* C, float* Q,
                       long long n, float dt, cudaStream_t st);

// Largest box around the grid centre (interior indices) where `damp` is zero,
// found and verified on the device; writes {z0, z1, x0, x1, y0, y1} into the
// device array `box` (7 ints: the 6 bounds and a verification word).
// Tiled 2D float32 stencil of one shot (sw_batch.cu), on the per-point
// coefficients of form_coefficients; 16-byte aligned pitched rows.
bool tiled2d_supported(const Layout& L);
// `zero_box` (z0, z1, x0, x1) bounds points where Q is known to be zero.
void tiled2d_launch(const Layout& L, bool vd, float* un, const float* uc, const float* up,
                    const float* C, const float* Q, const float* den,
                    const Weights<float>& W, const int* zero_box, cudaStream_t st);

// A 2D float32 shot's step parameters for the tiled stencil with
// owner-computes sources and boundary edges (sw_batch.cu): tiles of 16 x 128
// interior points; `fused` is set when the first and last tiles hold at
// least r + 1 rows and columns (then each tile can apply the sources and the
// boundary operations of its own points after its stencil, exactly).
struct Shot2D {
    Layout L;
    const float *C, *Q, *den, *vel, *damp;
    Weights<float> W;
    int zb[4];
    Windows<float> src;
    const float* wavelet;
    size_t wavelet_count;
    float dt;
    Windows<float> rec;
    float* receivers;
    int bc[4];
    int tiles_x, tiles_z, ntiles;
    int zoff;  // the 16-row tiles start zoff rows above the interior
    int fused;
};

// One shot of a multi-shot step launch (device memory): its step parameters,
// its level array and its ring (or null).
struct StepShot {
    Shot2D S;
    float* lev;
    float* ring;
};

// A time step of `nshots` fused shots of one layout in one launch:
// `per_shot` >= ntiles + receiver blocks (kThreads / 32 receivers a block)
// of the shot with the most receivers. Levels i_un, i_uc, i_up of each
// shot's level array (G elements each); with a ring, its row at element
// `ring_off`; with `record`, the receivers of u_cur into row n - 1.
void step2d_launch_shots(const StepShot* shots, int nshots, int per_shot, int r, bool vd,
                         long long G, int i_un, int i_uc, int i_up, long long n,
                         long long ring_off, bool record, cudaStream_t st);

// Fills `S`; false when the layout does not suit the tiled 2D kernel.
bool shot2d_prepare(Shot2D& S, const Layout& L, const float* C, const float* Q,
                    const float* den, const float* vel, const float* damp,
                    const Weights<float>& W, const int* zero_box, const Windows<float>& src,
                    const float* wavelet, size_t wavelet_count, float dt,
                    const Windows<float>& rec, float* receivers, const int* bc);

// Step n of `S` (fused only) in one launch: stencil, sources, edges and the
// record of u_cur. `ring` (optional, 2 (nx - 2r) + 2 (nz - 2r - 2) floats)
// receives the interior edge lines after the sources, before the boundary
// conditions: rows r and nz - r - 1, then columns r and nx - r - 1 without
// the corner rows.
void step2d_launch(const Shot2D& S, bool vd, float* un, const float* uc, const float* up,
                   long long n, cudaStream_t st, float* ring = nullptr);

// Every step of `S` in one cooperative launch (small grids, where per-step
// kernels are bound by their start-up): `slots` (device) holds the physical
// next/cur/prev slot of each step, `bar` two zeroed words for the grid
// barrier, `err` the run's status word. False when the device does not
// allow it (nothing launched).
bool persistent2d_launch(const Shot2D& S, bool vd, float* u, const int* slots, int steps,
                         long long begin, unsigned* bar, int* err, cudaStream_t st);

// gz = s1_z * sum_k c1_k (rho(z+k) - rho(z-k)) at interior points (3D).
void form_density_z(const float* den, float* gz, const Layout& L, const Weights<float>& W,
                    cudaStream_t st);
// Whether the selected 3D kernel reads gz (then the run forms it).
bool wants_density_z(const Layout& L, bool vd);

int kernel_policy();
void set_kernel_policy(int policy);
// The SIMWAVE_POLICY_* the tiled launch resolves `policy` to for radius r.
int resolve_policy(int policy, int r, bool vd);

// Kernels of sw_stencil_tmem.cu (SIMWAVE_POLICY_TMEM, _STAGE_RELEASE): x
// rows per CTA of a policy; the launch, false when the context or the radius
// does not suit it (then nothing is launched).
int tmem_rows(int policy);
bool tmem_launch(const TiledContext& ctx, int policy, bool vd, float* un, const float* uc,
                 const float* up, const float* coefC, const float* den, const Layout& L,
                 const Weights<float>& W, cudaStream_t st);
// Per-axis tables of the mask along the zero box's centre lines (device
// arrays of nz, nx, ny floats) and their check: *bad (device) becomes
// nonzero if a point with one axis outside the box differs from its table.
void damp_face_tables(const float* damp, const Layout& L, const int* box, float* tz,
                      float* tx, float* ty, int* bad, cudaStream_t st);

void find_zero_box(const float* damp, const Layout& L, int* box, cudaStream_t st);

}  // namespace sw
