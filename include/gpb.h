/*
 * gpb.h -- C ABI of libgpb, a GB300 (sm_103a) implementation of the gPb
 * contour stage of yanyp/UCM-MPI-GPU.
 *
 * It replaces the reference's engine boundary
 *     void computeGPb(unsigned rank, unsigned width, unsigned height,
 *                     unsigned* data, float** hostGPb, float** hostGPbAllConcat);
 *     int  getCudaDeviceCount();
 * (damascene/include/globalPb.h:35,44; called from src/globalPb.cpp:282 inside
 * GlobalPbCuda, src/globalPb.cpp:247-313).  Those two C++ symbols are also
 * exported with their original signatures and semantics (see gpb_damascene.h).
 *
 * Conventions
 *  - Input pixels are packed as data[y*width + x] = B<<16 | G<<8 | R
 *    (src/globalPb.cpp:264-276).
 *  - Every entry point returns a gpb_status and never throws.
 *  - A context owns its device buffers, stream and tables; it is reentrant per
 *    context and may be used from one host thread at a time.
 *  - Output buffers returned through float** are malloc()ed; release them with
 *    free() or gpb_free(), as the reference's caller does (src/globalPb.cpp:310).
 */
#ifndef GPB_H_
#define GPB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GPB_OK = 0,
  GPB_ERR_ARG = 1,       /* bad argument (size, NULL pointer, missing codebook) */
  GPB_ERR_CUDA = 2,      /* a CUDA runtime call failed                           */
  GPB_ERR_NOMEM = 3,     /* device or host allocation failed                     */
  GPB_ERR_NOCONV = 4,    /* the eigensolver hit its matvec cap                   */
  GPB_ERR_TIMEOUT = 5,   /* a bounded device wait gave up                        */
  GPB_ERR_INTERNAL = 6,  /* an unexpected host exception; the message says more  */
  GPB_ERR_TOO_LARGE = 7  /* image beyond gpb_texton_labels_static's fixed scratch, or a
                            batch whose padded vector layout reaches 2^31 entries */
} gpb_status;

typedef enum {
  /* gPb of the reference's CPU path (src/globalPb.cpp:128-245, fixes on):
   * orient planes [o][y][x] row-major, o = 0..7; nmax = max_o |gPb_o|. */
  GPB_COMPAT_CPU = 0,
  /* computeGPb output (damascene/src/damascene.cu:546-603): GPU weight sets,
   * nmax = max_o gPb_o where mPb > 0.05 (before the sigmoid), orient planes
   * sigmoid-rescaled, plane i = orientation {4,5,6,7,0,1,2,3}[i], each stored
   * column-major ([i*H*W + x*H + y]). */
  GPB_COMPAT_DAMASCENE = 1
} gpb_compat;

typedef enum {
  GPB_EIG_LANCZOS = 0,   /* plain cold-start thick-restart Lanczos (Krylov-Schur) */
  GPB_EIG_WARM = 1,      /* block Chebyshev-filtered solver warm-started from the
                            2x2-aggregated (coarse) problem                       */
  GPB_EIG_BLOCK = 2,     /* the same block solver from a seeded random start      */
  GPB_EIG_LEARNED = 3    /* the same block solver started from the learned
                            network's 32 fields (gpb_learned_set)                */
} gpb_eig_mode;

typedef struct {
  int device;            /* CUDA device ordinal, -1 = current                     */
  int compat;            /* gpb_compat                                            */
  int nvec;              /* eigenvectors, including the trivial one (9)           */
  float eig_tol;         /* Ritz residual tolerance on the unit eigenvectors      */
  int eig_max_matvecs;   /* cap per patch                                         */
  int krylov_dim;        /* Krylov-Schur basis size m                             */
  int krylov_keep;       /* vectors kept at a restart                             */
  int eig_mode;          /* gpb_eig_mode                                          */
  int keep_intermediates;/* 1: retain per-stage buffers for gpb_fetch(); 2: also counts */
  int cheb_degree;       /* Chebyshev filter degree of the block solver          */
  float warm_tol;        /* residual at which the coarse warm-start solve stops  */
  float eig_gap_frac;    /* block solvers: a patch also needs residual <= this x
                            its smallest gap between wanted eigenvalues (floor
                            1e-7; 0 disables; default 0.1)                       */
} gpb_params;

typedef struct gpb_ctx gpb_ctx;

/* one patch of a batch: a window of a packed image (row stride in pixels) */
typedef struct {
  uint32_t width, height;
  const uint32_t* packed_bgr;
  size_t stride;
} gpb_patch;

/* per-patch outputs; NULL members are malloc()ed by the library */
typedef struct {
  float* nmax;    /* H*W                  */
  float* orient;  /* 8*H*W (layout per compat) */
} gpb_result;

typedef struct {
  double ms_total, ms_h2d, ms_texton, ms_cues, ms_nms, ms_buildw, ms_eig, ms_spb, ms_d2h;
  long matvecs_max;           /* largest per-patch matvec count of the last call   */
  long matvecs_total;
  int restarts;
  float max_residual;         /* largest final Ritz residual                       */
  long texton_repaired;       /* pixels whose texton label went to the FP64 repair */
  int gpu_launches;           /* kernels launched by the last call                 */
  /* per-kernel timing of the eigensolver (filled when GPB_PROFILE=1 in the
   * environment at gpb_create): total ms, launches and algorithmic bytes */
  double spmv_ms, orth_ms;
  long spmv_launches, orth_launches;
  double spmv_bytes, orth_bytes;
  int eig_fallback;           /* 1: a block solver missed its target and the batch
                                 was solved again by plain Lanczos                 */
  int graph_replays;          /* launch chains of the last call replayed as CUDA
                                 graphs (stage chains, filters, Lanczos cycles)    */
} gpb_stats;

/* intermediates available through gpb_fetch() (keep_intermediates = 1) */
typedef enum {
  GPB_STAGE_TEXTON = 0,   /* uint8  H*W                              */
  GPB_STAGE_LABBINS = 1,  /* uint8  3*H*W (L, a, b bins)              */
  GPB_STAGE_MPB_O = 2,    /* float  8*H*W weighted cue sum per orient */
  GPB_STAGE_MPB = 3,      /* float  H*W   mPb after NMS and clip      */
  GPB_STAGE_W = 4,        /* float  H*W*81 symmetric affinities       */
  GPB_STAGE_EVALS = 5,    /* float  nvec                               */
  GPB_STAGE_EVECS = 6,    /* float  nvec*H*W unit eigvecs of A        */
  GPB_STAGE_SPB = 7,      /* float  8*H*W                              */
  GPB_STAGE_CUES = 8,     /* float  12*8*H*W raw cue maps             */
  GPB_STAGE_GPB_O = 9,    /* float  8*H*W gPb planes before layout    */
  /* uint8 H*W*4*4*32*32, keep_intermediates = 2: per pixel, annulus
   * (r <= 3, 5, 10, 20, cumulative), cue (L, a, b, texton), counter row
   * (half*16 + slice) and bin -- the raw half-disc histogram counts
   * (sum the two halves of a slice) */
  GPB_STAGE_COUNTS = 10,
  /* float H*W*9, gpb_warmnet_capture on: the first 9 columns of the
   * warm-start block (prolongated coarse Ritz vectors), pixel-major, before
   * the learned correction */
  GPB_STAGE_WARM0 = 11,
  GPB_STAGE_DEG = 12      /* float  H*W   affinity degree sum_q W(p,q) */
} gpb_stage;

void gpb_default_params(gpb_params* p);
gpb_status gpb_create(gpb_ctx** ctx, const gpb_params* p);
void gpb_destroy(gpb_ctx* ctx);

/* The 13 x K FP32 texton codebook (row f = Schmid filter f, column k =
 * codeword k), as src/SPFeatures.cpp:300-313 reads from
 * <piece>_texton_codebook.yml.  K <= 32. */
gpb_status gpb_set_codebook(gpb_ctx* ctx, const float* codebook, int K);
/* Same, parsed from an OpenCV YAML file holding "texton_codebook". */
gpb_status gpb_load_codebook_yml(gpb_ctx* ctx, const char* path);

/* One patch; *out_nmax (H*W) and *out_orient (8*H*W) are malloc()ed. */
gpb_status gpb_compute(gpb_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* packed_bgr,
                       float** out_nmax, float** out_orient);

/* n patches of any sizes (each side >= 32) in one batched pass. */
gpb_status gpb_compute_batch(gpb_ctx* ctx, const gpb_patch* patches, size_t n, gpb_result* out);

/* Device-resident variant: d_packed holds the patches back to back (patch i
 * at d_packed + offsets[i], tightly packed rows); results are written to
 * d_nmax / d_orient at the same offsets (orient: 8 planes per patch starting
 * at 8*offsets[i]).  Host arrays widths/heights/offsets have n entries. */
gpb_status gpb_compute_batch_device(gpb_ctx* ctx, size_t n, const uint32_t* widths,
                                    const uint32_t* heights, const size_t* offsets,
                                    const uint32_t* d_packed, float* d_nmax, float* d_orient);

/* Copy an intermediate of patch `patch` of the last call into dst. */
gpb_status gpb_fetch(gpb_ctx* ctx, int stage, size_t patch, void* dst, size_t dst_bytes);

gpb_status gpb_last_stats(gpb_ctx* ctx, gpb_stats* st);

/* The context's autotuner: for each shape bucket of a tunable kernel (the
 * texton tile's thread count, the block step's X staging and tile queue),
 * "key=chosen variant (median ms of each variant); ...", -1 while a bucket
 * is still being tried.  Every variant gives identical results; the first
 * launches of a bucket try them on real work.  GPB_NO_TUNE=1 in the
 * environment at gpb_create keeps the default variants.  Writes at most n
 * bytes including the terminating 0; returns the report's full length.  No
 * counterpart in the reference. */
size_t gpb_tuning_report(gpb_ctx* ctx, char* buf, size_t n);

/* Stitching the patches of the last compute call into whole-image planes on
 * the device; replaces Pieces2Gpb (src/utilities.cpp:180-213). */
typedef enum {
  GPB_STITCH_LAST = 0,      /* each patch's whole box, in patch order: later patches
                               overwrite the overlaps (the reference's rule)         */
  GPB_STITCH_INTERIOR = 1,  /* each patch writes only its interior box               */
  GPB_STITCH_BLEND = 2      /* overlaps averaged with weights falling linearly over
                               `ramp` pixels towards each patch edge inside the image */
} gpb_stitch_mode;

typedef struct {
  int32_t x0, y0;           /* the patch's top-left corner in the image              */
  int32_t ix, iy, iw, ih;   /* its interior box, in patch coordinates                */
} gpb_place;

/* n must be the patch count of the last gpb_compute* call on ctx, in the same
 * order.  d_nmax (width*height floats) and d_orient (8*width*height, plane
 * after plane) receive row-major image planes in the patch output's plane
 * order; pixels no patch covers are left as they were.  Device pointers;
 * synchronous on the context's stream.  BLEND uses a context buffer of
 * 10*width*height floats. */
gpb_status gpb_stitch_device(gpb_ctx* ctx, int mode, uint32_t width, uint32_t height, const gpb_place* places,
                             size_t n, int ramp, float* d_nmax, float* d_orient);

/* Per-superpixel descriptors for GLSVM (SPFeatures, src/SPFeatures.cpp) of
 * patch `patch` of the last compute call, from that call's texton map, grey
 * image and input colours.  d_labels: the patch's superpixel map (W*H int32,
 * row-major, device); pixels whose label is outside [0, n_labels) are
 * skipped.  d_out (device, n_labels rows of doubles) receives per row
 *   [ texton histogram (K columns, only if with_textons) |
 *     grey-level histogram, bin = grey / bin_step (255 / bin_step + 1 columns) |
 *     0 (the Harris corner descriptor's column, not computed) |
 *     mean B, G, R ]
 * histograms divided by the superpixel's size and multiplied by 10, means
 * multiplied by 10/255 (genTextonFeatures :260-275, genIntensityHistograms
 * :101-114, genAverageFeatures :380-391); rows of empty superpixels are zero.
 * Synchronous on the context's stream. */
gpb_status gpb_superpixel_features(gpb_ctx* ctx, size_t patch, const int32_t* d_labels, int32_t n_labels,
                                   int bin_step, int with_textons, double* d_out);

/* The reference's per-piece files (src/main.cpp:444-452), from host planes:
 * a rows x cols row-major matrix as an OpenCV FileStorage YAML matrix named
 * `name` with dt d (OpenCVFileWriter, src/utilities.cpp:33-37; values with
 * 17 significant digits), and as an 8-bit greyscale PNG scaled min..max to
 * 0..255 with round-to-nearest-even (OpenCVImageWriter, :21-31). */
gpb_status gpb_write_yml(const char* path, const char* name, const float* data, uint32_t rows, uint32_t cols);
gpb_status gpb_write_png_minmax(const char* path, const float* data, uint32_t rows, uint32_t cols);

/* Texton and Lab-bin labels of one image already on the device, computed
 * without allocating memory, on the device or the host.  No counterpart in
 * the reference: its texton stage (src/SPFeatures.cpp:277-360) allocates
 * its buffers on every call, and so do gpb_compute*, which grow the
 * context's buffers to each new batch shape.
 *
 * Meant for callers that cannot allocate at this point: a serving process
 * that has handed all device memory to its own pool, or one running work on
 * other streams that cannot take the device-wide synchronisation that
 * cudaMalloc / cudaFree may bring.
 *
 * d_packed  width x height pixels, B<<16 | G<<8 | R, rows tightly packed.
 * d_labels  width x height uint32, written as L | a<<8 | b<<16 | texton<<24
 *           (the bytes gpb_fetch returns for GPB_STAGE_LABBINS and
 *           GPB_STAGE_TEXTON after gpb_compute on the same image).
 * stream    a cudaStream_t, or NULL for the context's stream; the call only
 *           enqueues work on it.
 * Limits    each side >= 32; width * height <= 1,048,576 (2^20) pixels, in
 *           at most 8192 tiles of 16 x 16: a larger image returns
 *           GPB_ERR_TOO_LARGE and launches nothing.  Both pointers 4-byte
 *           aligned; the context needs a codebook.
 * Scratch   one fixed array of 9,568,768 bytes in the library's device code,
 *           one per device: the grey image, the tile list, the repair list
 *           and its counter.  The counter must be 0 when the texton kernel
 *           starts; the first kernel of every call writes it, so no call
 *           depends on what an earlier one left there.
 * First call on each device looks the array's address up
 *           (cudaGetSymbolAddress), which may load the library's device
 *           code: make it once before any stream capture.
 * Overlap   all calls on one device share the one array, so two calls whose
 *           work overlaps on the GPU (different streams or threads) race and
 *           give wrong labels: put them on one stream, or order them with
 *           events.  The kernels read the codebook from the device's constant
 *           tables; a later call of any context that reloads those tables
 *           (another codebook or compat mode) first waits, on the GPU, for
 *           this call's kernels.
 * Reset     the array's address is kept per device for the life of the
 *           process: do not call this entry point after a cudaDeviceReset
 *           of that device. */
gpb_status gpb_texton_labels_static(gpb_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* d_packed,
                                    uint32_t* d_labels, void* stream);

/* ---- Oriented watershed transform and ultrametric contour map ----------
 * Contours2Ucm (src/contours2ucm.cpp:405-490, called from
 * UCM_generator::generateUCM2, src/UCMgenerator.cpp:23-51), the consumer of
 * GlobalPbCuda's orientation planes.
 *
 * orient      8 planes of width x height floats, row-major, plane o being
 *             gPbOrient[o] as GlobalPbCuda returns it (after the sigmoid, in
 *             oriMap order); device memory when orient_on_device, else host.
 * double_size 1: ucm_out receives the (2H+1) x (2W+1) map of the doubled
 *             grid ("doubleSize", what main.cpp:457 asks for); 0: the
 *             (H+1) x (W+1) map of its even-even points.  Row-major doubles.
 * The quantisation, flooding, painting, super-contour grid, cleaning and
 * labelling run on the context's device; contour fitting and the greedy
 * merge on the calling thread.  Not reentrant per context. */
typedef struct {
  uint32_t n_regions;   /* regions of the finest partition              */
  uint32_t n_vertices;  /* vertices and edges of the fitted contours     */
  uint32_t n_edges;
  uint32_t n_artefacts; /* isolated zeros fixed by the cleaning step     */
  int32_t fit_ok;       /* 0: the chords could not be made consistent;
                           as in the reference nothing was painted      */
  double ms_front;      /* device: max, quantise, flood                  */
  double ms_fit;        /* host: contour fitting                         */
  double ms_mid;        /* device: paint, super contour, clean, label    */
  double ms_merge;      /* host: mean-boundary merge and calibration     */
  double ms_total;
} gpb_ucm_info;

gpb_status gpb_ucm(gpb_ctx* ctx, uint32_t width, uint32_t height, const float* orient, int orient_on_device,
                   int double_size, double* ucm_out, gpb_ucm_info* info);

/* The same for n images at once: the pieces the reference hands to one MPI
 * rank each (src/main.cpp:456-459).  They are flooded together (one CTA
 * each); their contour fitting and merging run on the context's host
 * threads, one image per thread.  widths, heights, orient and ucm_out have
 * n entries, info n entries or NULL.  The doubled grids of all images
 * together must stay below 2^31 cells. */
gpb_status gpb_ucm_batch(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                         const float* const* orient, int orient_on_device, int double_size, double* const* ucm_out,
                         gpb_ucm_info* info);

/* Intermediates of image `image` of the last gpb_ucm / gpb_ucm_batch call on
 * this context, copied to host:
 * GPB_UCM_QUANT   u8, H x W: the 8-bit max-over-orientations image
 * GPB_UCM_ARCS    u8, H x W: 1 on watershed pixels
 * GPB_UCM_WSWT    float, H x W: contour strength painted along the edges
 * GPB_UCM_WSWT2   float, (2H+1) x (2W+1): the cleaned doubled grid ws_wt2
 * GPB_UCM_REGIONS int32, H x W: region ids of the finest partition */
enum { GPB_UCM_QUANT = 0, GPB_UCM_ARCS = 1, GPB_UCM_WSWT = 2, GPB_UCM_WSWT2 = 3, GPB_UCM_REGIONS = 4 };
gpb_status gpb_ucm_fetch(gpb_ctx* ctx, size_t image, int what, void* host, size_t bytes);

/* The host stages, usable without a device.
 * gpb_ucm_fit_contours: fit_contour (src/fit_contour.cpp) of a 0/1 map of
 *   watershed arcs, row-major height x width (fewer than 2^31 pixels).
 *   Vertices as (row, column) pairs, edges as vertex-id pairs, each edge's
 *   interior pixels (row, column) in off[e] .. off[e+1]; completion edges
 *   are not produced.  Returns the number of edges, -1 for a bad argument
 *   or a capacity that is too small, -2 when the chords cannot be made
 *   consistent (the reference then returns no contours), -3 when host
 *   memory runs out.
 * gpb_ucm_mean_pb: UcmMeanPb (src/ucm_mean_pb.cpp:402-449): the
 *   (2H+1) x (2W+1) mean-boundary map (fewer than 2^31 points) from ws_wt2
 *   and the pixels' region ids (0-based; negative ids are skipped), all
 *   row-major.  GPB_ERR_NOMEM when host memory runs out.
 * gpb_ucm_labels_at_scale: UCM_generator::generateLabelsAtScaleK
 *   (src/UCMgenerator.cpp:120-161): regions of the doubled-grid map (fewer
 *   than 2^31 points) at threshold k, labels (0-based) of the height x width
 *   pixels; returns the number of regions, -1 for a bad argument or when
 *   host memory runs out. */
int32_t gpb_ucm_fit_contours(const uint8_t* bw, uint32_t width, uint32_t height, int32_t cap_vertices,
                             int32_t cap_edges, int32_t cap_pixels, int32_t* n_vertices, int32_t* vertices,
                             int32_t* edges, int32_t* off, int32_t* pixels);
gpb_status gpb_ucm_mean_pb(const double* ws_wt2, const int32_t* labels, uint32_t width, uint32_t height,
                           double* ucm);
int32_t gpb_ucm_labels_at_scale(const double* ucm2, uint32_t width, uint32_t height, double k, int32_t* labels);

/* ---- Learned correction of the warm start ------------------------------
 * A two-layer conv net (3 x 3 conv of the start block's first 9 columns and
 * mPb to 16 channels, ReLU, 1 x 1 conv to 9 corrections) refines the
 * prolongated coarse Ritz vectors before the fine block solve of
 * GPB_EIG_WARM.  Weights: W1 [16][10][9], b1 [16], W2 [9][16], b2 [9]
 * (GPB_WARMNET_PARAMS floats); NULL switches the correction off (the
 * default).  Training uses gpb_warmnet_grad_device: over n patches given
 * by their sizes and device arrays of normalised inputs x~ [Ntot][9],
 * mPb [Ntot] and targets v~ [Ntot][9] (concatenated patch after patch),
 * the mean squared error and its gradient for the given weights. */
#define GPB_WARMNET_PARAMS 1609
gpb_status gpb_warmnet_set(gpb_ctx* ctx, const float* weights, size_t n);
gpb_status gpb_warmnet_capture(gpb_ctx* ctx, int on);
gpb_status gpb_warmnet_grad_device(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                                   const float* d_xt, const float* d_mpb, const float* d_vt, const float* weights,
                                   double* loss, float* grad);

/* ---- Learned warm start (GPB_EIG_LEARNED) -----------------------------
 * A 4-level convolutional encoder-decoder maps each patch's mPb and
 * affinity degree (/81), per pixel, to 32 fields that start the block
 * eigensolver in place of a random block or the coarse-grid solve.  3 x 3
 * convolutions with channels 16/32/64/64 per level, 2 x 2 mean pooling,
 * nearest up-sampling with skip concatenation, ReLU, a 16 -> 32 head: BF16
 * weights and activations on the tensor cores, FP32 accumulation.  The
 * parameters (gpb_learned_nparams() FP32 values) are, per convolution in
 * the order e0a e0b e1a e1b e2a e2b e3a e3b d2a d2b d1a d1b d0a d0b head,
 * W[cout][3][3][cin] then b[cout].  Training minimises, per patch,
 * 9 - tr(V^T P_Y V): the energy of the 9 eigenvectors V the plain solver
 * finds outside the span of the 32 fields Y.  The solve itself still
 * iterates to eig_tol, and a block solve that fails falls back to plain
 * Lanczos.  No counterpart in the reference.
 *
 * The _device calls take n patches by their sizes and device arrays holding
 * them back to back: mPb and degree [H*W] each, targets V [H*W][9], fields
 * Y [H*W][32]. */
size_t gpb_learned_nparams(void);
/* the weights (n = gpb_learned_nparams()); NULL drops them */
gpb_status gpb_learned_set(gpb_ctx* ctx, const float* params, size_t n);
gpb_status gpb_learned_get(gpb_ctx* ctx, float* params, size_t n);
gpb_status gpb_learned_forward_device(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                                      const float* d_mpb, const float* d_deg, float* d_y);
/* the loss summed over the patches and its gradient (host, parameter layout) */
gpb_status gpb_learned_grad_device(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                                   const float* d_mpb, const float* d_deg, const float* d_v, double* loss,
                                   float* grad);
/* Adam (beta 0.9 / 0.999) on the context's weights over `epochs` passes of
 * the n patches in seeded random minibatches of `batch` patches; the mean
 * loss per patch of each epoch into loss_per_epoch (host, `epochs`). */
gpb_status gpb_learned_train_device(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                                    const float* d_mpb, const float* d_deg, const float* d_v, int batch, int epochs,
                                    float lr, uint64_t seed, double* loss_per_epoch);

int gpb_device_count(void);
const char* gpb_status_str(gpb_status s);
/* The message of the most recent failed call on the context ("" before
 * any); valid until the next call on the context. */
const char* gpb_last_error(const gpb_ctx* ctx);
void gpb_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* GPB_H_ */
