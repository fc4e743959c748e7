/*
 * gbsdf -- C ABI of the GB300 (sm_103a) neural-SDF field and volume-rendering path.
 *
 * Every entry point takes plain pointers to DEVICE memory (unless stated),
 * element counts, and the CUDA stream to run on (passed as void*; NULL = the
 * legacy default stream).  Nothing synchronises implicitly; nothing allocates
 * device memory: scratch buffers are passed in by the caller and their sizes are
 * reported by the *_workspace_size() queries.  Every call returns a status
 * (GBSDF_OK = 0); gbsdf_last_error() returns a thread-local message for the
 * last failing call on the calling thread.  Exceptions never cross this ABI.
 *
 * Reference interfaces replaced (paths inside NVlabs/neuralangelo):
 *   hash grid ............ tcnn.Encoding(3, {"otype": "HashGrid", ...})
 *                          projects/neuralangelo/utils/modules.py:42-50 (built), :84-86 (called)
 *   NeuS alpha ........... Model.compute_neus_alphas  projects/neuralangelo/model.py:275-298
 *   compositing .......... render.alpha_compositing_weights / composite
 *                          projects/nerf/utils/render.py:87-112
 *   fused field step ..... NeuralSDF.forward + compute_gradients + NeuralRGB.forward +
 *                          compute_neus_alphas + compositing + Trainer._compute_loss and
 *                          their autograd backward (modules.py:68-220, model.py:158-190,
 *                          trainer.py:40-52, misc.py:74-89)
 *   lattice SDF + MC ..... extract_mesh / LatticeGrid / marching_cubes
 *                          projects/neuralangelo/utils/mesh.py:25-49, 68-101, 119-133
 *   importance sampler ... Model.sample_dists_hierarchical + nerf_util.sample_dists_from_pdf
 *                          projects/neuralangelo/model.py:250-267, projects/nerf/utils/nerf_util.py:41-68
 */
#ifndef GBSDF_H
#define GBSDF_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBSDF_OK               0
#define GBSDF_ERR_ARG          1   /* bad pointer, size, stride or alignment */
#define GBSDF_ERR_UNSUPPORTED  2   /* configuration the kernels are not built for */
#define GBSDF_ERR_CUDA         3   /* a CUDA runtime call failed */
#define GBSDF_ERR_TIMEOUT      4   /* a bounded device-side wait ran out */

#define GBSDF_MAX_LEVELS 32

#define GBSDF_F32 0
#define GBSDF_F16 1

/* Level table of a multi-resolution hash grid (tcnn "HashGrid" semantics).
 * Filled by gbsdf_grid_init; read-only for every other call. */
typedef struct gbsdf_grid {
    int32_t  n_levels;            /* L */
    int32_t  n_features;          /* F: 1, 2, 4 or 8 */
    int32_t  log2_hashmap_size;   /* T = 2^log2_hashmap_size entries max per level */
    int32_t  base_resolution;
    float    per_level_scale;
    float    scale[GBSDF_MAX_LEVELS];        /* position scale of each level */
    uint32_t resolution[GBSDF_MAX_LEVELS];   /* grid points per axis */
    uint32_t size[GBSDF_MAX_LEVELS];         /* entries in the level */
    uint32_t hashed[GBSDF_MAX_LEVELS];       /* 1 = spatial hash, 0 = dense */
    uint64_t offset[GBSDF_MAX_LEVELS + 1];   /* first entry of each level; offset[L] = total */
} gbsdf_grid;

/* Library version (major*10000 + minor*100 + patch). */
int gbsdf_version(void);

/* Message of the last failing call on this thread ("" if none). */
const char* gbsdf_last_error(void);

/* Number of CUDA devices visible (0 without a GPU); never fails. */
int gbsdf_device_count(void);

/* Fill a level table.  Replaces the level setup inside tcnn's GridEncoding that
 * modules.py:42-50 configures (n_levels, n_features_per_level,
 * log2_hashmap_size, base_resolution, per_level_scale).  Host-only. */
int gbsdf_grid_init(gbsdf_grid* grid, int n_levels, int n_features, int log2_hashmap_size,
                    int base_resolution, float per_level_scale);

/* Hash-grid forward.  Replaces tcnn.Encoding.forward (modules.py:85).
 * x       [M,3] float32 positions in grid units [0,1] (modules.py:82-83)
 * table   [offset[L], F] entries, dtype GBSDF_F32 or GBSDF_F16
 * out     [M, L*F] level-major, dtype out_dtype; levels >= active_levels are
 *         written as 0 (the coarse-to-fine mask of modules.py:91-93). */
int gbsdf_hashgrid_fwd(const gbsdf_grid* grid, int active_levels, const float* x, int64_t M,
                       const void* table, int table_dtype, void* out, int out_dtype, void* stream);

/* Hash-grid backward.  Replaces the autograd backward of tcnn.Encoding
 * (the dL/dparams path; numerical-gradient mode never needs dL/dx).
 * d_out   [M, L*F] float32 ; d_table [offset[L], F] float32, ACCUMULATED into. */
int gbsdf_hashgrid_bwd(const gbsdf_grid* grid, int active_levels, const float* x, int64_t M,
                       const float* d_out, float* d_table, void* stream);

/* Absolute entry index of each (point, active level, corner), int64 [M, A, 8].
 * Exposes the index computation for bit-exact parity checks. */
int gbsdf_hashgrid_indices(const gbsdf_grid* grid, int active_levels, const float* x, int64_t M,
                           int64_t* indices, void* stream);

/* NeuS alpha, forward.  Replaces Model.compute_neus_alphas (model.py:275-292)
 * with _get_iter_cos (model.py:294-298).
 * ray_unit [R,3], sdf [R,N], grad [R,N,3], dists [R,N], far [R] (float32);
 * s_var: device pointer to the scalar log inverse standard deviation (model.py:64);
 * alpha [R,N] out. */
int gbsdf_neus_alpha_fwd(int64_t R, int64_t N, const float* ray_unit, const float* sdf, const float* grad,
                         const float* dists, const float* far, const float* s_var, float progress,
                         float anneal_end, float* alpha, void* stream);

/* NeuS alpha, backward: d_alpha [R,N] -> d_sdf [R,N], d_grad [R,N,3] (written),
 * d_s_var [1] (accumulated). */
int gbsdf_neus_alpha_bwd(int64_t R, int64_t N, const float* ray_unit, const float* sdf, const float* grad,
                         const float* dists, const float* far, const float* s_var, float progress,
                         float anneal_end, const float* d_alpha, float* d_sdf, float* d_grad, float* d_s_var,
                         void* stream);

/* Compositing weights w_i = a_i * prod_{j<i}(1-a_j), forward, FP32 log-space
 * transmittance.  Replaces render.alpha_compositing_weights (render.py:87-99).
 * alpha [R,N] -> weights [R,N]. */
int gbsdf_composite_weights_fwd(int64_t R, int64_t N, const float* alpha, float* weights, void* stream);

/* Backward of the compositing weights: d_weights [R,N] -> d_alpha [R,N]. */
int gbsdf_composite_weights_bwd(int64_t R, int64_t N, const float* alpha, const float* d_weights,
                                float* d_alpha, void* stream);

/* ---------------------------------------------------------------------------
 * Fused dense layer on the tcgen05 tensor cores (fp16 operands, fp32 accumulate):
 *     Y[:, 0:N] = epi(X[:, 0:K] * W^T + bias ; G)
 * Replaces one torch.nn.Linear + activation of the SDF feature layer
 * (projects/neuralangelo/utils/mlp.py:55-69) and of the colour MLP
 * (projects/nerf/utils/nerf_util.py:187-196), forward or input-gradient:
 *   epi 0 identity, 1 relu, 2 softplus(beta)           (forward; bias added)
 *   epi 3 acc*[G>0], 4 acc*(1-exp(-beta*G))             (backward through the
 *         previous layer's activation; G = its stored output; bias ignored)
 * X [M, ldx] fp16, W [N, K] fp16 row-major, bias [N] fp32 (may be NULL),
 * G [M, ldg] fp16, Y [M, ldy] fp16 (fp32 when y_f32 != 0).  K % 16 == 0,
 * K <= 512 (and the weight slice within shared memory), N % 64 == 0, ldx/ldg/ldy % 8 == 0, 16-byte aligned bases.
 * Xlo (optional): low fp16 half of X (X = Xhi + Xlo), multiplied as well;
 * Ylo (optional): receives the fp16 rounding residual of Y (Y = Yhi + Ylo).
 * The split pair carries a gradient through the colour MLP's input-gradient
 * chain at ~2^-22 relative precision on the fp16 tensor cores.  err:
 * optional device int set non-zero when a bounded device wait runs out. */
/* Launch shape of gbsdf_dense for layers of K input and N output columns (a tuning choice;
 * results are unchanged): n_tile output columns per CTA (64, 128 or 256; 0 = the built-in
 * rule) and ring slots of the A pipeline (3 to 6, capped by shared memory; 0 = as many as fit).
 * A small process-wide table (32 shapes); set it before launches that should use it. */
int gbsdf_dense_tune(int K, int N, int n_tile, int nslots);
/* Device workspace of gbsdf_dense: 0 bytes (the tiles are staged in shared memory). */
size_t gbsdf_dense_workspace_size(int64_t M, int K, int N);
int gbsdf_dense(int64_t M, int K, int N, const void* X, const void* Xlo, int ldx, const void* W,
                const float* bias, const void* G, int ldg, void* Y, void* Ylo, int ldy, int y_f32, int epi,
                float beta, int* err, void* stream);

/* ---------------------------------------------------------------------------
 * Fused SDF field (hash grid + SDF layer 0 + head + 6 numerical-gradient taps).
 * Replaces NeuralSDF.forward / compute_gradients (modules.py:68-95, 131-156),
 * MLPforNeuralSDF layer 0 and head (mlp.py:55-69), the outside overwrite
 * (model.py:163) and builds NeuralRGB's input tail (modules.py:209-213).
 * Samples are a flat array; ray of sample s = s / S (S > 0) or sample_ray[s].
 * fp16 tensors are passed as void*.  Field meanings are documented in
 * neuralangelo_gb300/csrc/field.cu. */
typedef struct gbsdf_field_args {
    int64_t Ns;
    int32_t S;
    int32_t ld_h0c;          /* row stride of h0c in elements (0 = 256); columns past 255 are not written */
    const int32_t* sample_ray;
    const float* center;
    const float* ray_unit;
    const float* dists;
    const uint8_t* outside;
    const int32_t* app_idx;
    gbsdf_grid grid;
    int32_t active;
    int32_t K0;
    const void* table;       /* fp16 [entries, F] */
    const void* w0e;         /* fp16 [256, K0] */
    const void* w0eT;        /* unused (the backward reads W0e from w0b); may be NULL */
    const void* w0b;         /* fp16 [256, K0 + 16]: w0e | position and bias columns as hi/lo pairs
                                (x hi, b hi, x lo, b lo, x-weight lo; see the x0ext tail) */
    const float* w0x;        /* [256, 3] */
    const float* b0;         /* [256] */
    const float* whead;      /* [256] */
    const float* bhead;      /* [1] */
    float beta, eps, two_eps, eps2, outside_val;
    float d_table_scale;     /* factor on the table-gradient contributions (0 = 1), e.g. 1 / loss scale */
    void* xc;                /* fp16 [Ns, ldxc] colour input; columns >= 256 written by the forward:
                                x, SH(d), normal, app, zeros, and 1 in the last column */
    int32_t ldxc;
    int32_t app_dim;
    const float* app_table;  /* [n_images, app_dim] */
    float* sdf;              /* [Ns] */
    float* grad;             /* [Ns, 3] */
    float* hess;             /* [Ns, 3] */
    void* h0c;               /* fp16 [Ns, 256] */
    const float* d_sdf;      /* [Ns]    backward inputs, loss-scaled */
    const float* d_grad;     /* [Ns, 3] */
    const float* d_hess;     /* [Ns, 3] */
    const float* d_xc;       /* [Ns, ld_dxc] gradient of the colour-input tail */
    int32_t ld_dxc;
    int32_t normal_col;
    const float* d_h0c;      /* [Ns, 256] gradient of the centre layer-0 activation */
    float* d_table;          /* [entries, F] accumulated */
    void* d_pre0;            /* fp16 [126 T, 256], T = ceil(Ns / 18) tiles, tile-major rows (backward) */
    void* x0ext;             /* fp16 [126 T, 2 K0 + 16] tile-major rows: features hi | x,y,z hi, 1,
                                x,y,z lo, 1, x,y,z hi, 0 x 5 | features lo; written by the forward,
                                read by the backward; 16-byte aligned (the MLP kernels load its rows
                                by TMA) */
    float* d_enc;            /* [126 T, K0] gradient of the encoder features (backward workspace) */
    float* d_whead;          /* [256] accumulated */
    float* d_bhead;          /* [1] accumulated */
    int32_t* err;            /* device flag for timed-out waits */
    float* d_w0;             /* [256, K0 + 16] accumulated layer-0 weight gradient: columns
                                [0, K0) the features (hi + lo), [K0, K0 + 16) the x0ext tail.
                                Non-NULL (K0 <= 64): the backward accumulates it itself and
                                leaves d_pre0 unused (may be NULL); NULL: it writes d_pre0 */
    void* h0c_lo;            /* optional fp16 [Ns, ld_h0c]: h0c's low half, so h0c + h0c_lo carries the
                                FP32 activation to ~2^-22 (NULL: not written) */
    void* xc_lo;             /* optional fp16 [Ns, ldxc]: the low half of the colour-input tail columns
                                (>= 256) the forward writes; 0 in the constant-1 column (NULL: not written) */
    void* d_pre0_lo;         /* optional fp16 [126 T, 256]: d_pre0's low half (backward without d_w0; the
                                layer-0 weight gradient is d_pre0^T x0ext + d_pre0_lo^T [x hi | tail]) */
    const float* d_table_scale_dev;  /* optional device scalar used in place of d_table_scale (e.g. the
                                        inverse of a loss scale the device updates) */
    float* found_inf;        /* optional: the scatter sets *found_inf = 1 when it reads a non-finite d_enc
                                value (the table gradient would be non-finite) */
    int32_t taps;            /* numerical-gradient stencil: 6 (or 0) = +-eps along each axis, 18 samples of
                                7 evaluations per 126-row tile (modules.py:132-156); 4 = the tetrahedral
                                stencil, 25 samples of 5 evaluations per 125-row tile (modules.py:157-175):
                                then eps = the tap displacement normal_eps / sqrt(3), two_eps = 4 eps and
                                eps2 = eps^2.  x0ext, d_enc and d_pre0 hold ceil(Ns / samples per tile)
                                tiles of rows. */
    int32_t pad_taps;
    unsigned long long* d_table_fix;  /* optional int64 [entries, F]: deterministic table scatter.  Each
                                         contribution is added as a 64-bit fixed-point integer (48
                                         fraction bits) with integer atomics, whose sum does not depend
                                         on the order they land in, then added into d_table: two runs
                                         give bit-identical table gradients (|sum| < 2^15).  The call
                                         clears the buffer itself.  NULL: FP32 vector atomics. */
    /* Launch shapes (tuning choices, results unchanged; 0 = the built-in default): */
    int32_t scatter_cpt;     /* table corners per pass of the scatter for 8-feature fields: 2, 4 or 8 */
    int32_t fwd_ctas;        /* CTAs per SM launched for the MLP forward: 1 or 2 */
} gbsdf_field_args;

/* Sizes of the caller-owned buffers of the field calls for Ns samples, K0 encoder columns, a
 * tap count (6, 4, or 0 = 6) and the deterministic scatter (grid needed then).  The calls
 * allocate nothing; a caller sizes x0ext, d_enc, d_w0 / d_pre0 (and d_pre0_lo) and d_table_fix
 * from these.  The colour-input, h0c and per-sample output buffers are [Ns, ...] as declared
 * in gbsdf_field_args. */
typedef struct gbsdf_field_workspace {
    int64_t rows;              /* rows of x0ext, d_enc and d_pre0: tiles x 126 (6 taps) or x 125 (4 taps) */
    size_t x0ext_bytes;        /* fp16 [rows, 2 K0 + 16] */
    size_t d_enc_bytes;        /* fp32 [rows, K0] */
    size_t d_w0_bytes;         /* fp32 [256, K0 + 16] when K0 <= 64 (in-kernel layer-0 weight gradient), else 0 */
    size_t d_pre0_bytes;       /* fp16 [rows, 256] for d_pre0 and again for d_pre0_lo when K0 > 64, else 0 */
    size_t d_table_fix_bytes;  /* int64 [entries, F] for the deterministic scatter, else 0 */
} gbsdf_field_workspace;
int gbsdf_field_workspace_size(int64_t Ns, int32_t K0, int32_t taps, int32_t deterministic,
                               const gbsdf_grid* grid, gbsdf_field_workspace* out);

size_t gbsdf_field_args_size(void);
/* Forward: hash-grid gather of the 7 evaluations into x0ext, then the MLP forward
 * (NeuralSDF.forward + compute_gradients, modules.py:68-74,132-156). */
int gbsdf_field_fwd(const gbsdf_field_args* args, void* stream);
/* Backward: the MLP backward into d_enc / d_pre0 / d_whead / d_bhead, then the table-
 * gradient scatter into d_table (the tcnn.Encoding backward behind modules.py:85). */
int gbsdf_field_bwd(const gbsdf_field_args* args, void* stream);
/* The same four kernels one at a time, in step order (gbsdf_field_fwd = encode +
 * mlp_fwd, gbsdf_field_bwd = mlp_bwd + scatter), so each can be timed on its own. */
int gbsdf_field_encode(const gbsdf_field_args* args, void* stream);
int gbsdf_field_mlp_fwd(const gbsdf_field_args* args, void* stream);
int gbsdf_field_mlp_bwd(const gbsdf_field_args* args, void* stream);
int gbsdf_field_scatter(const gbsdf_field_args* args, void* stream);

/* ---------------------------------------------------------------------------
 * Fused per-ray rendering forward + backward: NeuS alpha (model.py:275-298),
 * FP32 log-space transmittance and compositing (render.py:87-112), the L1
 * colour, eikonal and curvature losses (trainer.py:40-52, misc.py:74-89) and
 * their gradients with respect to every per-sample input, one warp per ray.
 * Ray r owns samples [ray_offsets[r], ray_offsets[r+1]) (or [r S, r S + S)). */
typedef struct gbsdf_render_args {
    int64_t R;
    int32_t S;
    int32_t pad0;
    const int64_t* ray_offsets;  /* [R + 1] when S == 0 */
    const float* ray_unit;       /* [R, 3] */
    const float* dists;          /* [Ns] */
    const float* far;            /* [R] */
    const uint8_t* outside;      /* [R] */
    const float* target;         /* [R, 3] */
    const float* s_var;          /* [1] */
    const float* sdf;            /* [Ns] */
    const float* grad;           /* [Ns, 3] */
    const float* hess;           /* [Ns, 3] */
    const float* rgbs;           /* [Ns, 3] */
    float anneal;                /* min(progress / anneal_end, 1) */
    float w_render, w_eik, w_curv;
    float l1_scale;              /* d L1 / d rgb = l1_scale * sign (3 / (3 R) for the reference) */
    float mean_scale;            /* 1 / (number of samples in the eikonal/curvature means) */
    float loss_scale;            /* multiplies every gradient output */
    int32_t pad1;
    float* rgb;                  /* [R, 3] out */
    float* weights;              /* [Ns] out (may be NULL) */
    float* d_rgbs;               /* [Ns, 3] out */
    float* d_sdf;                /* [Ns] out */
    float* d_grad;               /* [Ns, 3] out */
    float* d_hess;               /* [Ns, 3] out */
    float* d_s_var;              /* [1] accumulated */
    double* loss_sums;           /* [4] accumulated: l1 sum, eikonal sum, curvature sum, (unused) */
    int32_t* err;                /* device flag: 2 = a ray longer than 512 samples was skipped */
    /* Background NeRF samples composited after each ray's object samples (model.py:129-141):
     * n_bg per ray (0: none), alpha = 1 - exp(-sigma dt) with the last interval to 1e10
     * (render.py:68-84).  Object + background samples of a ray must number <= 512. */
    int32_t n_bg;
    int32_t ld_d_bg_pre;         /* row stride (elements) of d_bg_pre */
    const float* bg_dists;       /* [R, n_bg] */
    const float* bg_sigma;       /* [R, n_bg] density (softplus output) */
    const float* bg_rgbs;        /* [R, n_bg, 3] */
    float* bg_weights;           /* [R, n_bg] out (may be NULL) */
    float* d_bg_rgbs;            /* [R, n_bg, 3] out */
    void* d_bg_pre;              /* fp16 out, row s at s * ld_d_bg_pre: d loss / d density pre-activation */
    /* Evaluation outputs (Model.render_image / render_rays_object, model.py:90-114, 175-178),
     * each may be NULL.  forward_only = 1 skips the losses and the backward (every d_* output
     * and target may then be NULL). */
    int32_t forward_only;
    int32_t pad2;
    float* out_opacity;          /* [R]    sum of the object samples' weights */
    float* out_gradient;         /* [R, 3] sum of the object samples' weights x (unnormalised) gradient */
    float* out_dist;             /* [R]    sum of weights x distance over object and background samples */
    /* Optional device scalars read in place of the host fields above (NULL: the host fields):
     * dyn[0] loss_scale, dyn[1] anneal, dyn[2] w_curv.  A captured CUDA graph then follows a
     * loss scale that the device updates and a schedule that the host refreshes between replays. */
    const float* dyn;
} gbsdf_render_args;

size_t gbsdf_render_args_size(void);
int gbsdf_render_fused(const gbsdf_render_args* args, void* stream);
/* Device workspace of gbsdf_render_fused for R rays of S samples (0: ragged) and n_bg
 * background samples: 0 bytes -- a ray's alphas and transmittances live in its warp's shared
 * memory (up to 512 samples), every other buffer is an argument. */
size_t gbsdf_render_workspace_size(int64_t R, int32_t S, int32_t n_bg);

/* Last colour layer (H -> 3, sigmoid) forward: rgbs = sigmoid(Y W^T + b).
 * Replaces the last Linear + sigmoid of NeuralRGB (modules.py:215, nerf_util.py:187-196).
 * Y fp16 [Ns, ldy] (hidden width H <= 256, H % 8 == 0), W [3, H] fp32, b [3]. */
int gbsdf_rgb_head_fwd(int64_t Ns, const void* Y, int ldy, int H, const float* W, const float* b, float* rgbs,
                       void* stream);

/* Its backward: d_rgbs [Ns,3] -> d_pre = d_rgbs rgbs (1 - rgbs), optionally written to
 * d_pre [Ns, 8] fp16 (columns 0-2, rest 0; may be NULL), dZ = (d_pre W) * [Y > 0] as an
 * fp16 pair dZ = dZ_hi + dZ_lo [Ns, H] (dZ_lo may be NULL), d_b [3] accumulated, and the
 * head's weight gradient d_W [3, H] += d_pre^T Y accumulated (may be NULL). */
int gbsdf_rgb_head_bwd(int64_t Ns, const void* Y, int ldy, int H, const float* W, const float* rgbs,
                       const float* d_rgbs, void* d_pre, void* dZ, void* dZ_lo, float* d_b, float* d_W,
                       void* stream);

/* Appearance-embedding gradient: d_app[app_idx[r]] += sum over ray r's samples of
 * d_xc[s, col0 : col0 + app_dim] (fp32). */
int gbsdf_app_grad(int64_t R, int32_t S, const int64_t* ray_offsets, const int32_t* app_idx, const void* d_xc,
                   int ld_dxc, int col0, int app_dim, float* d_app, void* stream);

/* SDF at points (pts [M,3]) or on a lattice block (pts NULL: point m = (i, j, k)
 * x-major with coordinates ax[i], ay[j], az[k], nx*ny*nz == M), times sign.
 * Replaces NeuralSDF.sdf (modules.py:73-74) as called by extract_mesh
 * (mesh.py:33-35, sign -1 per scripts/extract_mesh.py:85) and by the sampler's
 * no-grad evaluations (model.py:238, 245).  Only the weight fields of args are
 * read (grid, active, K0, table, w0e, w0x, b0, whead, bhead, beta, err). */
int gbsdf_sdf_points(const gbsdf_field_args* args, int64_t M, const float* pts, const float* ax, const float* ay,
                     const float* az, int nx, int ny, int nz, float sign, float* out, void* stream);

/* Canonical marching-cubes case table (host-only): tri [256][16][3] edge ids
 * (-1 padded), count [256] triangles per configuration. */
int gbsdf_mc_table(int32_t* tri, int32_t* count);

/* Workspace bytes for gbsdf_mc_block on an nx x ny x nz block. */
size_t gbsdf_mc_workspace_size(int nx, int ny, int nz);

/* Marching cubes at iso of one block (vol [nx,ny,nz] float32 device, x-major),
 * vertices in world space V = index position * intv + origin (origin: 3 doubles,
 * HOST pointer), then the unit-sphere filter (mesh.py:119-148).
 * Replaces mcubes.marching_cubes + filter_points_outside_bounding_sphere.
 * V [V_cap, 3] double and F [F_cap, 3] int64 (device) must hold the worst case
 * (3 nx ny nz vertices, 5 (nx-1)(ny-1)(nz-1) faces); counts [2] (device) gets
 * the kept vertex and face counts.  workspace: gbsdf_mc_workspace_size bytes,
 * 256-byte aligned.  The first call on a device uploads the case table to
 * constant memory (make it before any stream capture). */
int gbsdf_mc_block(const float* vol, int nx, int ny, int nz, double iso, const double* origin, double intv,
                   void* workspace, size_t ws_bytes, double* V, int64_t V_cap, int64_t* F, int64_t F_cap,
                   int64_t* counts, void* stream);

/* ---------------------------------------------------------------------------
 * Background NeRF pieces of the fused step (projects/neuralangelo/utils/modules.py:232-311).
 * gbsdf_bg_encode: for the NB background samples of each of R rays (points c + d t at
 * dists [R, NB]) writes the first layer's fp16 input row X [R NB, ldx] -- x/|x|, 1/|x|,
 * their 10-level Fourier code (nerf_util.py:134-147), a constant 1 at column 84, zeros up
 * to x_cols -- and the colour MLP's input tail T [R NB, ldt] -- SH(d) (16), the appearance
 * code app_table[app_idx[r]] (app_dim, may be 0), a constant 1, zeros up to t_cols.
 * X_lo / T_lo (optional, same row strides): the fp16 low halves, so X + X_lo and T + T_lo carry
 * the FP32 values to ~2^-22 (0 in the constant-1 and zero columns).
 * gbsdf_bg_density: sigma [M] = softplus((H + H_lo) [M, ldh] . w [H] + b[0]) (beta 1, threshold
 * 20); H_lo, the optional low half of H, has H's row stride. */
int gbsdf_bg_encode(int64_t R, int32_t NB, const float* center, const float* ray_unit, const float* dists,
                    const float* app_table, const int32_t* app_idx, int32_t app_dim, void* X, void* X_lo,
                    int32_t ldx, int32_t x_cols, void* T, void* T_lo, int32_t ldt, int32_t t_cols, void* stream);
int gbsdf_bg_density(int64_t M, const void* H, const void* H_lo, int32_t ldh, int32_t Hdim, const float* w,
                     const float* b, float* sigma, void* stream);

/* ---------------------------------------------------------------------------
 * Mesh output stage (scripts/extract_mesh.py:96-97 after utils/mesh.py:121-129 and
 * :43-46): optional vertex weld (coordinates equal after round-half-even of v *
 * weld_mult, e.g. 1e8 for trimesh's 8-digit merge; first occurrence kept), then
 * V * scale + offset, then faces re-indexed and those whose two heights
 * 2A/|v1-v0|, 2A/|v2-v0| are not both > min_side dropped (min_side 0: only faces that
 * repeat a vertex index; min_side < 0: none, as trimesh's per-block merge keeps them).  V [nv,3] float64 and F [nf,3] int64 are device
 * inputs; V_out [>= nv,3], F_out [>= nf,3] device outputs; counts [2] (vertices,
 * faces) device int64.  The caller owns a 256-byte aligned device workspace of
 * gbsdf_mesh_finalize_workspace_size(nv, nf) bytes.  err (device int, optional) gets
 * 3 if a hash probe ran past the table, 4 for a face index outside [0, nv). */
size_t gbsdf_mesh_finalize_workspace_size(int64_t nv, int64_t nf);
int gbsdf_mesh_finalize(const double* V, int64_t nv, const int64_t* F, int64_t nf, int weld, double weld_mult,
                        double scale, const double* offset, double min_side, void* workspace,
                        size_t workspace_bytes, double* V_out, int64_t* F_out, int64_t* counts, int* err,
                        void* stream);

/* Marching cubes of one block without any device allocation (no counterpart in
 * the reference).  For callers that cannot allocate device memory -- a host
 * application that owns the device budget and forbids allocations after
 * start-up, or a latency-critical loop where cudaMalloc/cudaFree could
 * synchronise the device.  Same inputs, outputs and results as gbsdf_mc_block,
 * but the scratch lives in a fixed 12.5 MiB file-scope device array of this
 * library, so blocks are limited to 33 x 33 x 33 points (larger ones are
 * rejected with GBSDF_ERR_ARG).  The first call on a device looks up the
 * array's device address (make it before any stream capture).  All calls share
 * the array: calls that overlap on the GPU race and must be serialised. */
int gbsdf_mc_block_noalloc(const float* vol, int nx, int ny, int nz, double iso, const double* origin, double intv,
                           double* V, int64_t V_cap, int64_t* F, int64_t F_cap, int64_t* counts, void* stream);

/* ---------------------------------------------------------------------------
 * Hierarchical importance sampler (the no-grad pre-pass placing the training
 * samples): Model.sample_dists_all / sample_dists_hierarchical
 * (projects/neuralangelo/model.py:232-267), nerf_util.sample_dists and
 * sample_dists_from_pdf (projects/nerf/utils/nerf_util.py:20-68).
 * Per-ray lists are rows of [R, ld] float32 arrays, updated in place. */
#define GBSDF_SAMPLER_MAX_LIST 512

typedef struct gbsdf_sampler_args {
    int64_t R;                 /* rays */
    int32_t ld;                /* row stride of dists / sdfs (>= the longest list) */
    int32_t n_list;            /* entries already in each row */
    int32_t n_merge;           /* fine samples of the previous round sorted in first (0..32) */
    int32_t n_fine;            /* new distances to draw (0 = merge only) */
    float   inv_s;             /* sharpness of this round: 64 * 2^h (model.py:240) */
    int32_t robust;            /* 1: interval slope = min(previous, current) (model.py:256-258) */
    const float* center;       /* [R, 3] camera centres */
    const float* ray_unit;     /* [R, 3] unit directions */
    float* dists;              /* [R, ld] sample distances (in / out) */
    float* sdfs;               /* [R, ld] their SDF values (in / out); NULL once no round needs them */
    const float* merge_d;      /* [R, n_merge] previous fine distances (may alias fine_d) */
    const float* merge_s;      /* [R, n_merge] their SDF values (read when sdfs != NULL) */
    float* fine_d;             /* [R, n_fine] new distances (out) */
    float* fine_pts;           /* [R * n_fine, 3] their points c + d t (out), or NULL */
} gbsdf_sampler_args;

size_t gbsdf_sampler_args_size(void);

/* Stratified coarse distances dists[r, k] = (u[r, k] + k) / n * (far - near) + near
 * for k < n (nerf_util.sample_dists, nerf_util.py:20-38; u NULL = 0.5, the
 * non-stratified case) and their points pts [R * n, 3] (or NULL).
 * Reads R, ld, center, ray_unit, dists of args; near, far [R]. */
int gbsdf_sampler_coarse(const gbsdf_sampler_args* args, int n, const float* u, int ldu, const float* near,
                         const float* far, float* pts, void* stream);

/* One hierarchical round (model.py:237-247, 250-267): sort the previous round's
 * n_merge fine samples into each row (concatenate + sort, SDF values follow),
 * then draw n_fine distances by inverting the CDF of the NeuS interval weights
 * at sharpness inv_s (FP32 visibility product, nerf_util.py:41-68).  With
 * n_fine = 0 the call only merges (the final round). */
int gbsdf_sampler_round(const gbsdf_sampler_args* args, void* stream);

/* Weight gradient of a dense layer on the tensor cores (the autograd weight gradient of
 * torch.nn.Linear behind nerf_util.py:187-196, mlp.py:55-69 and modules.py:268-284):
 * dW [N, K] (row stride ldw) = (accumulate ? dW : 0) + (dZ + dZ_lo)[M, N]^T X[M, K].
 * dZ, the optional low half dZ_lo (same strides) and X are fp16 row-major; FP32
 * accumulation and output.  N, K <= 512; the bias gradient is the column of X holding a
 * constant 1.  err: device flag set when a bounded wait times out (may be NULL). */
int gbsdf_wgrad(int64_t M, int N, int K, const void* dZ, const void* dZ_lo, int ldz, const void* X, int ldx,
                float* dW, int ldw, int accumulate, int* err, void* stream);

/* Gradients of weight-normalised linears (torch.nn.utils.weight_norm, dim 0: W = g v / ||v||
 * per output row; applied at projects/neuralangelo/utils/mlp.py:42-43 and
 * projects/nerf/utils/nerf_util.py:177-178) from the gradient of the effective weight, with the loss scale taken off; replaces
 * autograd's per-layer weight-norm backward.  An entry with v == NULL is plain: the weight's
 * gradient gets s dW and the bias's s db (s = *scale_dev when scale_dev is not NULL, else scale).
 * Gradient tensors (dv, dg, dbias) are contiguous; acc_* = 1 adds into them, 0 overwrites.
 * Up to GBSDF_WN_MAX_LAYERS entries per call, one launch. */
#define GBSDF_WN_MAX_LAYERS 16
typedef struct gbsdf_weightnorm_layer {
    int64_t rows, cols;
    const float* dW;      /* effective-weight gradient [rows, cols], row stride ld_dw */
    int64_t ld_dw;
    const float* db;      /* bias gradient [rows], element stride ld_db, or NULL */
    int64_t ld_db;
    const float* v;       /* weight_v [rows, cols] contiguous, or NULL for a plain entry */
    const float* g;       /* weight_g [rows] */
    float* dv;            /* weight_v.grad (plain: weight.grad) [rows, cols] */
    float* dg;            /* weight_g.grad [rows] */
    float* dbias;         /* bias.grad [rows], or NULL */
    int32_t acc_v, acc_g, acc_b, pad;
} gbsdf_weightnorm_layer;
int gbsdf_weightnorm_bwd(int32_t n, const gbsdf_weightnorm_layer* layers, const float* scale_dev, float scale,
                         void* stream);
size_t gbsdf_weightnorm_layer_size(void);   /* sizeof(gbsdf_weightnorm_layer), for binding checks */

/* Working copies of weight-normalised (or plain) weights for the fused step: per entry, rows of
 * W = g v / ||v|| (the norm over all `cols` of each source row; g == NULL: W = v), columns
 * [col0, col0 + ncols), written to any of: dst16 (fp16, row stride ld16, the segment's first
 * column at dst16), dst16_lo (fp16 residual W - fp16(W), dst16's layout), dst16T (fp16
 * transposed: element (r, j) at dst16T[j * ldT + r]), dst32 (FP32, row stride ld32).  Replaces
 * the weight-norm forward of each linear (the reference's weight property) and the casts,
 * transposes and column reorders of the packing.  Up to GBSDF_WN_MAX_LAYERS entries, one launch. */
typedef struct gbsdf_weightnorm_pack {
    int64_t rows, cols;
    const float* v;       /* weight_v or the plain weight, [rows, ld_src] */
    int64_t ld_src;
    const float* g;       /* weight_g [rows], or NULL for a plain weight */
    int64_t col0, ncols;
    void* dst16;
    int64_t ld16;
    void* dst16_lo;
    void* dst16T;
    int64_t ldT;
    float* dst32;
    int64_t ld32;
} gbsdf_weightnorm_pack;
int gbsdf_weightnorm_fwd(int32_t n, const gbsdf_weightnorm_pack* entries, void* stream);
size_t gbsdf_weightnorm_pack_size(void);

/* Self-test of the bounded waits (no counterpart in the reference): one GPU thread waits on an
 * mbarrier with the limit timeout_ns (0 to 2 s); nothing arrives on it unless arrive_first.
 * status [2] int32 (device): status[0] = 1 when the wait ran out, 0 when it completed;
 * status[1] = the wait's wall time in microseconds.  Every kernel's waits on TMA, MMA and
 * pipeline barriers end the same way: after the limit they set the caller's err flag and the
 * kernel returns, so a stalled pipeline surfaces as a status instead of a hung GPU. */
int gbsdf_selftest_wait(int64_t timeout_ns, int arrive_first, int* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBSDF_H */
