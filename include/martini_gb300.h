/*
 * martini_gb300 -- C ABI of the GB300 source-insertion library.
 *
 * The library inserts SPH particles into a spectral data cube, i.e. it
 * computes for every pixel (i, j) and channel c
 *
 *     cube[i][j][c] = sum_p  W_p(i, j) * S_p(c)                  [Jy / pix^2]
 *
 * where W_p is the SPH kernel integrated over pixel (i, j) and S_p the
 * particle's channel spectrum.  This is MARTINI's
 * ``Martini.insert_source_in_cube`` (reference: martini/martini.py:285-407)
 * with the per-pixel contraction of ``_BaseMartini._evaluate_pixel_spectrum``
 * (martini/martini.py:243-283), the kernel pixel integrals
 * ``_BaseSPHKernel._px_weight`` / ``_kernel_integral``
 * (martini/sph_kernels.py:85-119, :400-441, :544-685, :791-858, :994-1044,
 * :1136-1165, :1330-1363, :1486-1564) and the spectra of
 * ``_BaseSpectrum.init_spectra`` (martini/spectral_models.py:63-200,
 * :386-425, :544-570).  The reference is pure Python and has no FFI; these
 * entry points are what a ctypes/cffi binding of ``_insert_source_in_cube``
 * calls.
 *
 * Conventions
 *   - All array pointers are DEVICE pointers owned by the caller.
 *   - Every call is asynchronous on the given stream unless stated.
 *   - Return value: MG_OK or a negative MG_ERR_* code; a message for the
 *     last error of the calling thread is available from mg_last_error().
 *   - The cube layout is [i][j][c] (x = RA index slowest, channel fastest),
 *     float32, the padded grid of the reference's DataCube._array.
 */
#ifndef MARTINI_GB300_H
#define MARTINI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MG_OK 0
#define MG_ERR_INVALID_ARGUMENT (-1)
#define MG_ERR_CUDA (-2)
#define MG_ERR_WORKSPACE (-3)      /* workspace too small for this problem */
#define MG_ERR_NOT_MONOTONIC (-4)  /* channel edges not strictly monotonic */
#define MG_ERR_UNSUPPORTED (-5)
#define MG_ERR_TIMEOUT (-6)        /* a bounded device-side wait expired */

/* SPH kernel types (martini/sph_kernels.py) */
#define MG_KERNEL_WENDLAND_C2 0   /* _WendlandC2Kernel      :340-478   */
#define MG_KERNEL_WENDLAND_C6 1   /* _WendlandC6Kernel      :481-721   */
#define MG_KERNEL_CUBIC_SPLINE 2  /* _CubicSplineKernel     :724-894   */
#define MG_KERNEL_QUARTIC_SPLINE 3 /* _QuarticSplineKernel  :1402-1600 */
#define MG_KERNEL_GAUSSIAN 4      /* _GaussianKernel(trunc) :897-1080  */
#define MG_KERNEL_DIRAC 5         /* DiracDeltaKernel       :1083-1204 */

/* spectral models (martini/spectral_models.py) */
#define MG_SPECTRUM_GAUSSIAN 0    /* GaussianSpectrum  :304-485 */
#define MG_SPECTRUM_DIRAC 1       /* DiracDeltaSpectrum :488-587 */
#define MG_SPECTRUM_TABLE 2       /* caller-supplied spectra[n][nc] (any model) */

/* contraction forms */
#define MG_FORM_FP32 0            /* FP32 CUDA-core contraction */
#define MG_FORM_BF16X3 1          /* BF16 hi+lo split, three tcgen05 products (~16 bits per
                                     operand: about 1e-5 relative per term, below the
                                     1e-5-of-peak / 1e-6-of-flux bar only on average) */
#define MG_FORM_F16X3 2           /* FP16 hi+lo split (power-of-two scaled), three tcgen05 products */
#define MG_FORM_BF16X6 3          /* BF16 hi+mid+lo split (exact for FP32 operands: 24 bits in
                                     three 8-bit pieces), six tcgen05 products (every cross term
                                     down to 2^-16 relative); the chosen tensor-core form */

#define MG_MAX_KERNELS 4

typedef struct mg_kernel_spec {
  int32_t type;      /* MG_KERNEL_* */
  float truncate;    /* Gaussian truncation in sigma (MG_KERNEL_GAUSSIAN only) */
} mg_kernel_spec;

/*
 * One insertion problem: particles already projected to pixel coordinates
 * (the state the reference holds after Martini.__init__: source.pixcoords,
 * sph_kernel.sm_lengths/_rescale/sm_ranges/kernel_indices, spectral inputs).
 */
typedef struct mg_problem {
  int64_t n;                   /* particle count (may be 0) */
  const double* x;             /* [n] pixel coordinate on axis 0 (0-based, padded) */
  const double* y;             /* [n] pixel coordinate on axis 1 */
  const double* sm_range;      /* [n] footprint half-width, px (sph_kernel.sm_ranges) */
  const float* h_eff;          /* [n] sm_lengths * _rescale, px */
  const int8_t* kernel_index;  /* [n] index into kernels[], -1 means kernels[0]; NULL = all 0 */
  int32_t n_kernels;           /* 1..MG_MAX_KERNELS */
  mg_kernel_spec kernels[MG_MAX_KERNELS];

  int32_t spectral_model;      /* MG_SPECTRUM_* */
  const double* v;             /* [n] line-of-sight velocity, km/s (GAUSSIAN/DIRAC) */
  const float* sigma;          /* [n] Gaussian width, km/s, or NULL to use sigma_const */
  float sigma_const;
  const double* amp;           /* [n] mHI / D^2 / 2.36e5 (Jy km/s) (GAUSSIAN/DIRAC) */
  const float* spectra;        /* [n][nc] Jy (TABLE only) */

  int32_t nx, ny, nc;          /* padded cube size */
  int32_t padx, pady;          /* pad on each side (flux sums skip it) */
  const double* edges;         /* [nc+1] channel edges, km/s, strictly monotonic */
  float* cube;                 /* [nx][ny][nc] output, Jy / pix^2, overwritten */
  double* flux;                /* optional [nc+1]: total flux (Jy), then per channel; NULL = skip */
  int32_t form;                /* MG_FORM_* */
  int32_t accumulate;          /* 0: cube is overwritten; 1: the insertion is added to
                                  the cube's contents (the reference's _array +=,
                                  martini/martini.py:338); flux then sums the result */
} mg_problem;

/* sizes reported by mg_plan */
typedef struct mg_plan_info {
  int64_t n_pairs;          /* (tile, particle) pairs after footprint binning */
  int64_t n_items;          /* reserved (0) */
  int64_t n_partial_items;  /* upper bound on split-K partial tiles */
  int64_t n_tiles;
  size_t workspace_bytes;   /* mg_workspace_size(p, n_pairs, n_partial_items), plus the
                               spectrum store of the tensor-core forms (Gaussian lines) */
} mg_plan_info;

/* Library version string. */
const char* mg_version(void);

/* Message for the last error returned on the calling thread. */
const char* mg_last_error(void);

/*
 * Workspace bytes needed for a problem of this shape with room for
 * max_pairs (tile, particle) pairs and max_partial_items split-K partial
 * tiles (the counts mg_plan reports).
 */
int mg_workspace_size(const mg_problem* p, int64_t max_pairs, int64_t max_partial_items,
                      size_t* bytes);

/*
 * Bin the particles and report the exact pair/item counts and the workspace
 * size mg_insert needs.  Needs a workspace of at least
 * mg_workspace_size(p, 0, 0).  SYNCHRONISES the stream (it reads the counts
 * back).  Returns MG_ERR_NOT_MONOTONIC if the channel edges are not strictly
 * monotonic.
 */
int mg_plan(const mg_problem* p, void* workspace, size_t workspace_bytes, void* stream,
            mg_plan_info* info);

/*
 * Full insertion: footprint binning, spectra, kernel weights, contraction,
 * cube write and (if p->flux) the FP64 flux sums.  Asynchronous on stream;
 * no host synchronisation and no allocation, so it can be captured in a
 * CUDA graph.  The workspace must have been sized by mg_workspace_size with
 * the same max_pairs / max_partial_items.  If the data need more than that,
 * the device code skips the contraction and mg_check() returns
 * MG_ERR_WORKSPACE.  Bytes beyond mg_workspace_size(p, max_pairs,
 * max_partial_items) hold the per-particle spectrum store of the tensor-core
 * forms (Gaussian lines, computed once per particle instead of once per
 * tile); mg_plan's workspace_bytes has room for it.  With less room the
 * lines are evaluated inside the contraction: same results, slower.
 */
int mg_insert(const mg_problem* p, void* workspace, size_t workspace_bytes, int64_t max_pairs,
              int64_t max_partial_items, void* stream);

/* stages of mg_insert_stages (bit mask) */
#define MG_STAGE_BIN 1        /* records, tile histogram, plan, tile-major list */
#define MG_STAGE_CONTRACT 2   /* cube clear, contraction, split-K reduction */
#define MG_STAGE_FLUX 4       /* FP64 flux sums (if p->flux) */
#define MG_STAGE_SPEC 8       /* per-particle spectrum store (tensor-core forms, Gaussian
                                 lines; runs between BIN and CONTRACT; a BIN stage
                                 invalidates it, and CONTRACT then evaluates in-kernel) */
#define MG_STAGE_ALL 15

/*
 * mg_insert restricted to some stages, in the order BIN, SPEC, CONTRACT,
 * FLUX, on the same workspace (a stage reads what the previous ones left
 * there).  For timing stages
 * separately; mg_insert == mg_insert_stages(..., MG_STAGE_ALL, ...).
 */
int mg_insert_stages(const mg_problem* p, void* workspace, size_t workspace_bytes,
                     int64_t max_pairs, int64_t max_partial_items, int32_t stages, void* stream);

/*
 * Batches: several cubes in one insertion (a survey of many galaxies).  No
 * counterpart in the reference, which inserts one source per Martini object
 * (martini/martini.py:827-861); a population is a loop over Martini objects.
 * Every problem of a batch must share the kernel table, spectral model,
 * contraction form and accumulate flag; each has its own particles, cube,
 * channel grid and flux.  One launch sequence bins all cubes together and
 * one persistent contraction kernel works through all their tiles from a
 * single queue, so small cubes do not pay a pipeline each.  The per-cube
 * table is written to the workspace by kernels (no host copies), so a batch
 * insertion can be captured in a CUDA graph.  Semantics otherwise as the
 * single-problem calls (which are batches of one).  At most 65535 cubes.
 */
int mg_workspace_size_batched(const mg_problem* probs, int32_t nprob, int64_t max_pairs,
                              int64_t max_partial_items, size_t* bytes);
int mg_plan_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                    size_t workspace_bytes, void* stream, mg_plan_info* info);
int mg_insert_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                      size_t workspace_bytes, int64_t max_pairs, int64_t max_partial_items,
                      void* stream);
int mg_insert_stages_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                             size_t workspace_bytes, int64_t max_pairs, int64_t max_partial_items,
                             int32_t stages, void* stream);

/*
 * Launch shape of an insertion and its autotuner.  No counterpart in the
 * reference, whose only scheduling knob is the pixel thread pool
 * (martini/martini.py:344-362).  mg_tune times the contraction of the
 * caller's own problem under every candidate shape and caches the fastest
 * for the problem's class: form, kernel table, spectral model, number of
 * cubes, widest band, particle count (octave) and mean (tile, particle)
 * pairs per tile (half octave, from max_pairs).  mg_insert* then use the
 * cached shape of their class (the default when none is cached).  The cache
 * is per process and guarded by a mutex; it holds the only mutable
 * library-wide state besides per-device attribute caches.
 */
typedef struct mg_tuning {
  int32_t kc;            /* particles per tensor-core stage: 0 = the form's default
                            (64), or 32 (tensor-core forms) */
  int32_t items_per_sm;  /* work items per SM (split-K granularity), 1..24; 0 = 24 */
  int32_t cost_order;    /* 1: work queue ordered by estimated cost, largest first;
                            0: segment (tile) order */
  int32_t reserved;
} mg_tuning;

/* The default launch shape: kc 0, 6 items per SM, cost order. */
void mg_tuning_default(mg_tuning* out);

/* Candidate shapes mg_tune times for a form: up to cap into out; returns
 * how many there are. */
int mg_tuning_candidates(int32_t form, mg_tuning* out, int32_t cap);

/*
 * Autotune: for every candidate shape bin the problem (batch) and time its
 * contraction stage `reps` times with CUDA events on the stream; cache the
 * fastest (smallest median) for the problem's class and return it in *best
 * (and its time in *best_ms, if not NULL).  Same workspace contract as
 * mg_insert.  SYNCHRONISES the stream.  Runs with accumulate off, so it
 * OVERWRITES the cubes: call it before the insertion whose result is kept.
 */
int mg_tune_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                    size_t workspace_bytes, int64_t max_pairs, int64_t max_partial_items,
                    int32_t reps, void* stream, mg_tuning* best, float* best_ms);
int mg_tune(const mg_problem* p, void* workspace, size_t workspace_bytes, int64_t max_pairs,
            int64_t max_partial_items, int32_t reps, void* stream, mg_tuning* best,
            float* best_ms);

/* The cached shape of this problem's class: 1 and *out when cached, 0 and
 * the default when not.  Host only (no GPU access). */
int mg_tuning_lookup(const mg_problem* probs, int32_t nprob, int64_t max_pairs, mg_tuning* out);

/* Cache a shape for this problem's class (e.g. one tuned in an earlier run).
 * Host only.  Returns MG_ERR_INVALID_ARGUMENT for a shape the form cannot
 * run. */
int mg_tuning_store(const mg_problem* probs, int32_t nprob, int64_t max_pairs,
                    const mg_tuning* t);

/* Forget every cached shape. */
void mg_tuning_reset(void);

/*
 * GPU set-up: what Martini.__init__ does on the host before the insertion,
 * in FP64 on the GPU.  Per particle: sky position, distance and line-of-sight
 * velocity (martini/sources/sph_source.py:265-326), TAN projection to pixel
 * coordinates and the spectral pixel (sph_source.py:328-362), smoothing
 * length in pixels (martini/sph_kernels.py:235-262), adaptive kernel choice,
 * footprint range (sph_kernels.py:1241-1274, :257-262), amplitude
 * mHI / D^2 / 2.36e5 and thermal width (spectral_models.py:127-145, :465-485),
 * then the reference's pruning (martini/martini.py:168-241).  The kept
 * particles are written in their original order to `out`, ready for
 * mg_problem.  Asynchronous; the kept count is written to out->n_kept.
 */
typedef struct mg_source {
  int64_t n;
  const double* xyz;          /* [n][3] kpc, rotation already applied */
  const double* vxyz;         /* [n][3] km/s */
  const double* hsm;          /* [n] smoothing lengths, kpc */
  const double* mHI;          /* [n] Msun */
  const double* T;            /* [n] K (thermal widths) or NULL */
  double ra, dec;             /* source position, deg */
  double distance;            /* Mpc */
  double vpeculiar;           /* km/s */
  double h;                   /* Hubble flow h (v = h * 100 km/s/Mpc * r) */
} mg_source;

typedef struct mg_grid {
  double crpix[3];            /* 1-based reference pixels (datacube.py:438-486), padded */
  double cdelt[3];            /* deg, deg, and km/s (VRAD) or Hz (FREQ) */
  double crval[3];            /* deg, deg, and km/s or Hz */
  int32_t freq_mode;          /* 1: spectral axis in frequency */
  int32_t nx, ny, nc;         /* padded spatial sizes, channels */
  double px_size_arcsec;
  double max_channel_width;   /* max |dv| of the channel edges, km/s (pruning) */
} mg_grid;

typedef struct mg_kernel_choice {
  int32_t n_kernels;          /* 1, or the adaptive tuple's length (<= 4) */
  int32_t adaptive;           /* 1: index of the first valid kernel, -1 if none */
  int32_t upper[4];           /* validity: 0: h * rescale >= threshold; 1: <= (DiracDelta) */
  double threshold[4];
  double rescale[4];
  double size_in_fwhm[4];
} mg_kernel_choice;

#define MG_PRUNE_SPATIAL 1
#define MG_PRUNE_SPECTRAL 2
#define MG_PRUNE_MASS 4
#define MG_PRUNE_ALL 7

typedef struct mg_particles {  /* device arrays with room for n particles */
  double* x;
  double* y;
  double* sm_range;
  float* h_eff;
  int8_t* kernel_index;       /* NULL unless adaptive */
  double* v;                  /* km/s */
  float* sigma;               /* thermal widths (NULL unless src->T) */
  double* amp;                /* mHI / D^2 / 2.36e5 */
  int64_t* n_kept;            /* device scalar */
} mg_particles;

size_t mg_setup_workspace_size(int64_t n);
int mg_setup(const mg_source* src, const mg_grid* grid, const mg_kernel_choice* kc,
             int32_t spectral_model, float sigma_const, int32_t prune, const mg_particles* out,
             void* workspace, size_t workspace_bytes, void* stream);

/*
 * Global profile: the spatially integrated spectrum of a source, in Jy
 * (GlobalProfile.insert_source_in_spectrum, martini/martini.py:1551-1596:
 * every particle that survives spectral and mass pruning contributes its
 * whole line).  Uses p->n, v, sigma / sigma_const, amp, spectral_model (GAUSSIAN
 * or DIRAC), nc and edges; the spatial fields are ignored.  spectrum[nc] is
 * FP64 on the device.  Deterministic (fixed summation order).  Asynchronous;
 * mg_check(workspace) reports non-monotonic channel edges.
 */
size_t mg_global_profile_workspace_size(int64_t n, int32_t nc);
int mg_global_profile(const mg_problem* p, double* spectrum, void* workspace,
                      size_t workspace_bytes, void* stream);

/*
 * Beam convolution (Martini.convolve_beam, martini/martini.py:863-901):
 * out = scale * (cube (*) kernel) in "same" mode per channel (the reference's
 * scipy fftconvolve of each spatial slice), over the unpadded pixels only,
 * with zeros outside the padded cube.  cube: device [nx][ny][nc] (padded),
 * kernel: device [kx][ky] (odd sizes, pads >= half sizes), out: device
 * [nx - 2 padx][ny - 2 pady][nc].  scale converts Jy/arcsec^2 to Jy/beam
 * (the beam area in arcsec^2).  FP32 accumulation.  Asynchronous.
 */
int mg_convolve_beam(const float* cube, int32_t nx, int32_t ny, int32_t nc, int32_t padx,
                     int32_t pady, const float* kernel, int32_t kx, int32_t ky, float scale,
                     float* out, void* stream);

/*
 * Read back the device status word of the last mg_plan/mg_insert on this
 * workspace (SYNCHRONISES the stream).  Returns MG_OK, MG_ERR_WORKSPACE,
 * MG_ERR_NOT_MONOTONIC or MG_ERR_TIMEOUT.
 */
int mg_check(void* workspace, void* stream);

/*
 * Materialise the spectra of a GAUSSIAN/DIRAC problem: out[n][nc] in Jy,
 * the reference's spectral_model.spectra (spectral_models.py:63-147).
 */
int mg_spectra(const mg_problem* p, float* out, void* stream);

/*
 * Flux sums of a cube already in device memory, returned in FP64 (each
 * pixel row summed in double-float, rows and channels in FP64, in a fixed
 * order): flux[0] = total over the unpadded region, flux[1 + c] = per
 * channel (martini/martini.py:367-392).
 */
int mg_flux(const float* cube, int32_t nx, int32_t ny, int32_t nc, int32_t padx,
            int32_t pady, double* flux, void* workspace, size_t workspace_bytes,
            void* stream);

/*
 * Size of the scratch array built into the library for mg_insert_noalloc
 * (held on every GPU that loads the library until the process exits).
 */
#define MG_NOALLOC_SCRATCH_BYTES ((size_t)128 << 20)

/*
 * mg_insert without a caller workspace.  No counterpart in the reference:
 * it exists for callers that cannot allocate GPU memory (code inside a
 * framework or memory pool that owns every device allocation, or paths where
 * an allocation is not allowed).  The scratch is a file-scope device array of
 * MG_NOALLOC_SCRATCH_BYTES; a problem whose fixed workspace part alone is
 * larger is rejected before any GPU work, and one whose binning turns out to
 * need more pairs or split-K tiles than the array holds returns
 * MG_ERR_WORKSPACE with a message naming the built-in scratch.  Every call
 * looks up the array's device address on the current device (nothing is
 * cached, so a device reset cannot leave a stale address).  Calls share the
 * array: calls that overlap on the GPU race.  Every call synchronises the
 * stream (it reads the status word back), so no call can be captured in a
 * CUDA graph.  Allocates nothing.
 */
int mg_insert_noalloc(const mg_problem* p, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MARTINI_GB300_H */
