/*
 * rdxg.h -- C ABI of the GB300 MOMFBD per-patch solver core.
 *
 * A drop-in for the per-patch work of redux's momfbd::Solver
 * (include/redux/momfbd/solver.hpp:86-179 in ISP-SST/redux): the caller (the job/worker
 * layer, unchanged) hands over the static job data that redux keeps in GlobalData (modes,
 * pupil, supports, constraint null space) once, then batches of patches (the float32
 * image cutouts of PatchData), and receives the mode coefficients, metric histories and
 * per-patch reports that Solver::run stores back into PatchData.
 *
 * Plain pointers and sizes only; every function returns an rdxg_status and never throws.
 * All host pointers are read or written synchronously before the call returns unless the
 * function says otherwise.  One handle per host thread; each handle owns one CUDA stream.
 */
#ifndef RDXG_H
#define RDXG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    RDXG_OK = 0,
    RDXG_ERR_ARG = 1,          /* bad argument or shape */
    RDXG_ERR_UNSUPPORTED = 2,  /* size not supported by the compiled kernels */
    RDXG_ERR_CUDA = 3,         /* CUDA runtime error (message in rdxg_last_error) */
    RDXG_ERR_STATE = 4,        /* call out of order (e.g. solve before set_patches) */
    RDXG_ERR_NONFINITE = 5,    /* non-finite metric or gradient */
    RDXG_ERR_NOMEM = 6
} rdxg_status;

typedef enum { RDXG_FP32 = 0, RDXG_FP64 = 1 } rdxg_precision;

/* gradient methods: the reference's analytic gradient (Vogel weights), the exact
 * derivative of the metric, and the reference's one-sided finite differences */
typedef enum { RDXG_GRAD_VOGEL = 0, RDXG_GRAD_EXACT = 1, RDXG_GRAD_FD = 2 } rdxg_grad_method;

typedef struct rdxg_solver rdxg_solver;

/* Geometry of a job: sizes that redux derives in MomfbdJob/Object::initProcessing. */
typedef struct {
    int32_t otf_size;      /* N = 2 * pupil_pixels (Solver::otfSize) */
    int32_t pupil_pixels;  /* n (job.pupilPixels) */
    int32_t patch_size;    /* image size; must equal otf_size */
    int32_t n_modes;       /* M */
    int32_t n_objects;
    int32_t n_images;      /* I: all images of all objects/channels of one patch */
    int32_t n_channels;    /* C: all channels of all objects */
    int32_t tilt_x;        /* index of the x-tilt mode (ModeSet::tiltMode.x), -1 if none */
    int32_t tilt_y;
    int32_t n_free;        /* columns of the null-space map (Constraints::nFreeParameters) */
    int32_t cutout_size;   /* image cutout size incl. the max-local-shift margins */
    int32_t max_patches;   /* batch capacity */
    int32_t precision;     /* rdxg_precision (RDXG_FP64 takes otf_size <= 88) */
    int32_t device;        /* CUDA device ordinal */
    int32_t eval_chunk;    /* images of one object per work item of the fused evaluation, 1..32
                              (0: 6).  The chunks' sums are added in a fixed order, so a patch's
                              results depend on this value (at the level of FP32 rounding) and on
                              nothing else of the batch.  Larger values (fewer, longer work
                              items) pay when several handles are solved together by
                              rdxg_solve_many and each handle has about one object per SM; small
                              ones when one handle holds the batch. */
} rdxg_geometry;

/* Static inputs (host pointers, copied by rdxg_create). */
typedef struct {
    const double* modes;          /* [M][n][n], already scaled by 1/lambda (GlobalData::get) */
    const double* pupil;          /* [n][n] Pupil */
    int32_t n_pupil_support;
    const int32_t* pupil_support; /* Pupil::pupilSupport, indices into n*n */
    int32_t n_otf_support;
    const int32_t* otf_support;   /* Pupil::otfSupport, indices into the centred N*N OTF */
    const int32_t* image_object;  /* [I] object of each image (images of an object contiguous) */
    const int32_t* image_channel; /* [I] global channel index of each image */
    const double* phi_fixed;      /* [C][n][n] Channel::phi_fixed (diversity) */
    const double* object_weight;  /* [nObj] Object::weight */
    const double* object_grad_step; /* [nObj] GRADDIFF_STEP * wavelength (SubImage::grad_step) */
    const double* window;         /* [ps][ps] Solver::window */
    const double* noise_window;   /* [ps][ps] Solver::noiseWindow */
    int64_t ns_nnz;               /* Constraints::ns_entries: alpha[row] += val * beta[col] */
    const int32_t* ns_rows;
    const int32_t* ns_cols;
    const double* ns_vals;
    const double* tilt_jacobian;  /* [2][2] ModeSet::J_T_xy (alpha -> pixel shift), or NULL */
} rdxg_static;

/* Solver settings (GlobalCfg fields read by Solver::run, config.hpp:196-228). */
typedef struct {
    int32_t mode_start;        /* MODE_START */
    int32_t mode_step;         /* MODE_STEP */
    int32_t max_iterations;    /* MAX_ITER */
    int32_t min_iterations;    /* MIN_ITER */
    int32_t target_iterations; /* N_DONE_ITER */
    int32_t fd_first;          /* 1: first gradient by finite differences (the reference) */
    int32_t max_metrics;       /* capacity of the per-patch metric history */
    int32_t check_every;       /* rounds between host checks for completion (0: 8) */
    double ftol;               /* FTOL */
    double eps;                /* EPS */
} rdxg_solve_params;

/* Per-patch outcome (what Solver::run logs and stores in PatchData). */
typedef struct {
    double initial_metric;
    double final_metric;       /* PatchData::finalMetric */
    int32_t iterations;        /* total CG iterations */
    int32_t status;            /* 0 ok, 1 gave up after too many failures */
    int32_t n_f_evals;         /* metric evaluations */
    int32_t n_df_evals;        /* gradient evaluations */
    int32_t fail_count;
    int32_t n_metrics;         /* entries of the metric history (PatchData::metrics) */
} rdxg_patch_report;

int rdxg_version(void);

/* Replaces Solver::Solver + Solver::init (solver.cpp:63-181). */
int rdxg_create(const rdxg_geometry* geometry, const rdxg_static* statics, rdxg_solver** out);
int rdxg_destroy(rdxg_solver* h);
const char* rdxg_last_error(const rdxg_solver* h);

/* FIT_PLANE (the RF_FIT_PLANE run flag): before the images are windowed, subtract the plane
 * fitted to the mean of each object's images, refit it when an object's images are
 * re-shifted, and add it back to the restored object (Object::fitAvgPlane, object.cpp:
 * 553-594; SubImage::getWindowedImg, subimage.cpp:106-150; Object::restorePatch,
 * object.cpp:410-413).  Loaded patches are prepared again. */
int rdxg_set_fit_plane(rdxg_solver* h, int32_t enable);

/* Work on a caller-provided CUDA stream (cudaStream_t); NULL restores the handle's own. */
int rdxg_set_stream(rdxg_solver* h, void* cuda_stream);

/* Loads a batch of patches: Channel::initPatch + Solver::shiftAndInit(alpha_offset, true)
 * (channel.cpp:846-953, solver.cpp:583-605, subimage.cpp:155-209).
 * cutouts: [P][I][cutout][cutout] float32 (PatchData channel images);
 * residual_alpha: [P][I][2] (y, x) channel residual tilt coefficients or NULL;
 * fixed_gamma: [P][nObj] regularisation overriding the noise-derived one, or NULL. */
int rdxg_set_patches(rdxg_solver* h, int32_t n_patches, const float* cutouts,
                     const double* residual_alpha, const double* fixed_gamma);

/* Same, with the cutouts already in device memory (no host copy). */
int rdxg_set_patches_device(rdxg_solver* h, int32_t n_patches, const float* d_cutouts,
                            const double* residual_alpha, const double* fixed_gamma);

/* Ragged batches: patches of one OTF size whose frames per channel and mode counts differ
 * (redux runs each such patch in the job of its own geometry, momfbdjob.cpp:576-591, with
 * that job's Constraints, constraints.cpp:536-622).  A shape gives the frames per channel
 * (each channel's first `frames` images of the handle, in its image order; every channel of
 * the handle must have the same number), the number of modes (the first n_modes of the
 * handle's mode set) and that geometry's null-space map, rows indexed image * n_modes + mode
 * over the shape's own images.  patch_shape[p] picks the shape of patch p; the next
 * rdxg_set_patches must load n_patches patches, each with its images in the first slots of
 * its [I] cutouts (the rest are ignored), and alpha arrays keep the [P][I][M] layout with
 * zeros in the slots and modes a patch does not use.  Each patch is solved exactly as by a
 * handle of its own geometry (the same evaluations, chunks, sums and maps).  n_shapes = 0
 * returns to uniform batches.  Not with REG_ALPHA weights or rdxg_metric_noalloc. */
typedef struct {
    int32_t frames;
    int32_t n_modes;
    int32_t n_free;
    int64_t ns_nnz;
    const int32_t* ns_rows;
    const int32_t* ns_cols;
    const double* ns_vals;
} rdxg_patch_shape;
int rdxg_set_patch_shapes(rdxg_solver* h, int32_t n_shapes, const rdxg_patch_shape* shapes, int32_t n_patches,
                          const int32_t* patch_shape);

/* Warm start (INIT_FILES): the initial mode coefficients [P][I][M] of the loaded patches,
 * the alpha_offset that Solver::loadInit fills from ObjectData::alpha (solver.cpp:412,
 * 726-733; Object::getInit, object.cpp:446-456), or NULL to start at zero.  As
 * Solver::shiftAndInit(alpha_offset, true) (solver.cpp:413, 584-605) the patches are prepared
 * again with every image's window shifted by the integer part of its initial tilt
 * (SubImage::adjustShifts, subimage.cpp:444-480), and every following solve starts from these
 * coefficients.  Call after rdxg_set_patches / rdxg_set_patches_device (which start at zero). */
int rdxg_set_initial_alpha(rdxg_solver* h, const double* alpha);

/* Continuation: every following solve starts from the coefficients [P][I][M] (as
 * alpha_offset, beta = 0) with the images as loaded, not re-cut -- the next iterations of a
 * solve whose images were never re-shifted (all modes at once), e.g. an FP64 handle taking
 * over an FP32 solution.  NULL starts at zero again.  The reference's Solver::run continues
 * within one stage the same way (alpha_offset fixed, beta from zero, solver.cpp:446); it
 * has no entry point for it. */
int rdxg_set_start_alpha(rdxg_solver* h, const double* alpha);

/* REG_ALPHA: weights [I][M] (the same for every patch) of the regularisation term
 * 0.5 sum alpha^2 w that Solver::metric adds to the metric (solver.cpp:804-811), the
 * reference's Solver::regAlphaWeights = REG_ALPHA / wavelength * nTotalPixels / atm_rms^2
 * (solver.cpp:147-156); NULL turns it off (REG_ALPHA = 0, the default).  As in
 * Solver::gradient (solver.cpp:860-885) the gradient starts from alpha * w and the enabled
 * modes are then assigned the data term, so alpha * w remains for the modes not yet enabled. */
int rdxg_set_reg_alpha(rdxg_solver* h, const double* weights);

/* Metric of every patch at alpha [P][I][M] (Solver::applyAlpha + Solver::metric,
 * solver.cpp:219-225, 763-817).  metric: [P]. */
int rdxg_metric(rdxg_solver* h, const double* alpha, double* metric);

/* Metric at alpha [P][I][M] evaluated the way the solver's line search does: with the
 * reference object of the batched metric taken at alpha_ref (the last gradient point) instead
 * of alpha.  Same result as rdxg_metric up to rounding; used to check that rounding. */
int rdxg_metric_with_reference(rdxg_solver* h, const double* alpha_ref, const double* alpha, double* metric);

/* rdxg_metric without any allocation.  No counterpart in the reference (its Solver::metric
 * works on buffers allocated per patch).  Same kernels, same work-item order and the same
 * result as rdxg_metric; every temporary of the evaluation (alpha, mode-expanded phases,
 * per-chunk accumulators, per-tile sums, work lists, per-patch metrics) lives in one
 * file-scope static device array of 16 MiB instead of buffers of the handle, and the work
 * lists are built on the device, so the call makes no device or host allocation (no
 * cudaMalloc, cudaFree or heap allocation).  For callers that cannot allocate: a process
 * whose caching allocator (e.g. PyTorch's) already holds nearly all device memory, where a
 * raw cudaMalloc fails or forces the cache to be emptied, and latency-critical loops where
 * cudaMalloc/cudaFree would synchronize the device and stall other streams.
 * Limits: the fused FP32 path only (OTF size 32, 64 or 88 with a symmetric OTF support;
 * otherwise RDXG_ERR_UNSUPPORTED), and a batch whose temporaries exceed 16 MiB (about 600 KB
 * per patch at N = 88 with 36 images and 36 modes, i.e. at most 26 such patches) is rejected
 * with RDXG_ERR_UNSUPPORTED and a message giving the sizes.  The handle's device must be the
 * current device.  rdxg_create looks up the array's address in the current context
 * (cudaGetSymbolAddress) and keeps it in the handle; with lazy module loading that lookup is
 * also what loads the array, so its 16 MiB are reserved when the handle is created and the
 * call itself neither loads nor allocates anything.  The address belongs to the context the
 * handle was created in (the device's primary context, as for every other call); a handle does
 * not survive cudaDeviceReset.  The scratch is shared by every handle on the device: calls that
 * overlap in time (from two threads, or on two streams) race on it and must be serialized by
 * the caller. */
int rdxg_metric_noalloc(rdxg_solver* h, const double* alpha, double* metric);

/* Gradient in alpha space [P][I][M] at alpha (Solver::my_df without the constraint map,
 * solver.cpp:228-234, 860-894); enabled: [M] flags or NULL (all); metric: [P] or NULL. */
int rdxg_gradient(rdxg_solver* h, const double* alpha, const uint8_t* enabled, int32_t method,
                  double* grad, double* metric);

/* Restored objects of every patch at alpha [P][I][M]: Object::restorePatch
 * (object.cpp:278-334) for the object image, with the Scharmer filter (image/utils.cpp:
 * 334-392) unless no_filter (RF_NO_FILTER); FP64 on the device.  frequency_cutoff: [nObj]
 * Object::frequencyCutoff (pupil.cpp:87; the filter cuts at 0.9 of it).  objects:
 * [P][nObj][patch_size][patch_size] float32 (ObjectData::img). */
int rdxg_restore(rdxg_solver* h, const double* alpha, const double* frequency_cutoff, int32_t no_filter,
                 float* objects);

/* rdxg_restore with the other outputs of Object::restorePatch (object.cpp:335-410, the
 * SF_SAVE_PSF / SF_SAVE_PSF_AVG / SF_SAVE_COBJ / SF_SAVE_RESIDUAL flags), FP64 on the device,
 * stored as float32 and trimmed to patch_size like the object (the fitted plane, with
 * FIT_PLANE, is added to the object after them, as the reference does):
 *   RDXG_RESTORE_PSF      psf [P][I][ps][ps]      SubImage::getPSF of every image
 *   RDXG_RESTORE_PSF_AVG  psf [P][nObj][ps][ps]   their mean per object (takes precedence)
 *   RDXG_RESTORE_COBJ     cobj [P][I][ps][ps]     SubImage::convolveImage of the float object
 *   RDXG_RESTORE_RESIDUAL res [P][I][ps][ps]      convolved object minus the image
 * Images are in the order of the geometry (objects' channels, frames).  Buffers for flags not
 * set may be NULL. */
#define RDXG_RESTORE_PSF 1
#define RDXG_RESTORE_PSF_AVG 2
#define RDXG_RESTORE_COBJ 4
#define RDXG_RESTORE_RESIDUAL 8
int rdxg_restore_ex(rdxg_solver* h, const double* alpha, const double* frequency_cutoff, int32_t no_filter,
                    int32_t outputs, float* objects, float* psf, float* cobj, float* res);

/* Full per-patch solve (Solver::run, solver.cpp:330-580) for every loaded patch.
 * alpha_out: [P][I][M]; reports: [P]; metrics: [P][max_metrics] or NULL. */
int rdxg_solve(rdxg_solver* h, const rdxg_solve_params* params, double* alpha_out,
               rdxg_patch_report* reports, double* metrics);

/* Same, leaving the results on the device; rdxg_fetch_results copies them out. */
int rdxg_solve_async(rdxg_solver* h, const rdxg_solve_params* params);
int rdxg_fetch_results(rdxg_solver* h, double* alpha_out, rdxg_patch_report* reports,
                       double* metrics);

/* Solver::run for the patches of several handles at once, e.g. one handle per patch
 * geometry (OTF size, frames, modes) of an uneven batch: the rounds of every handle are
 * captured into one CUDA graph, one branch per handle forked from the first handle's stream
 * (give each handle its own stream for the branches to run concurrently), and the graph is
 * launched until no handle has an active patch.  Every handle's results are then read with
 * rdxg_fetch_results; they are the same as those of rdxg_solve on that handle alone.  All
 * handles on one device, each listed once. */
int rdxg_solve_many(rdxg_solver* const* handles, int32_t n, const rdxg_solve_params* params);

/* Number of kernel launches issued by the last rdxg_solve / rdxg_solve_async. */
int64_t rdxg_last_launch_count(const rdxg_solver* h);

/* Mode expansion phi = phi_fixed + sum_m alpha_m Z_m of FP32 handles (SubImage::calcPhi /
 * addToPhi, subimage.cpp:509-544) on the tensor cores (tcgen05, FP32 accumulation) with the FP32
 * operands split into BF16 parts: mode 3 (the default) three parts (6xBF16 products, FP32-like:
 * metric, OTF and gradient within 1e-6 of FP64), mode 2 two parts (3xBF16: phases within ~1e-5
 * of their magnitude, gradients within ~3e-5); mode 0 on the CUDA cores in FP32 (on the general
 * path, OTF size 128, inside the transform kernel).  FP64 handles expand the modes inside their
 * transform kernel and only accept mode 0 (RDXG_ERR_STATE otherwise).  rdxg_phase_mode returns
 * the mode in use (0, 2 or 3). */
int rdxg_set_phase_mode(rdxg_solver* h, int32_t mode);
int32_t rdxg_phase_mode(const rdxg_solver* h);

/* Recomputed transforms.  The reference keeps every image's pupil function and OTF
 * (SubImage::PF, SubImage::OTF, subimage.hpp:156-158) from the metric evaluation to the
 * gradient (calcVogelWeight, subimage.cpp:348-371).  With on = 1 the handle keeps neither: the
 * gradient kernels form PF, its transform X and (where the evaluation keeps no full OTF, the
 * fused FP32 path) the OTF again from the phases: 16 N^2 + 8 n^2 bytes per image in FP32
 * (32 N^2 + 16 n^2 in FP64) are not held, and 8 N^2 more on the fused path, at the price of
 * one or two more transforms per gradient image.  rdxg_create chooses it by itself when keeping the transforms
 * of max_patches patches would exceed the device's free memory (RDXG_MEMORY_BUDGET in the
 * environment: a budget in bytes for the handle instead; RDXG_RECOMPUTE=0/1 forces it).
 * Results agree with the kept form to rounding (the general path bit for bit).  The
 * restoration then holds the batch's OTFs only during its call.  rdxg_recompute returns the
 * mode in use. */
int rdxg_set_recompute(rdxg_solver* h, int32_t on);
int32_t rdxg_recompute(const rdxg_solver* h);

/* Times the per-image and per-object kernels on the loaded batch at the current point with
 * CUDA events on the handle's stream: ms[0] forward (metric evaluation), ms[1] per-object
 * accumulation, ms[2] forward (gradient evaluation, also keeps the transforms), ms[3]
 * analytic adjoint gradient, ms[4] finite-difference gradient; average ms per launch over
 * reps launches.  Used to pick kernel shapes and to report the roofline. */
int rdxg_profile_kernels(rdxg_solver* h, int32_t reps, double* ms);

/* Launch shapes: threads per block of the kernels that dominate a round.  eval_threads: the
 * fused evaluation k_eval (512 or 384; 0 on the general path); forward_threads: the general
 * path's transform kernel k_forward (256 or 512, 512 or 1024 at OTF size 128; 0 on the fused
 * path); adjoint_threads: the analytic gradient k_adjoint (same choices as forward).  No
 * block size changes a result: every element is computed by the same arithmetic. */
typedef struct {
    int32_t eval_threads;
    int32_t forward_threads;
    int32_t adjoint_threads;
    /* radix plans of the same kernels' transforms: the first radix of the two-stage plan
     * (32: 8 or 4, 64: 8 or 16, 88: 8, 128: 16 or 8).  Unlike the block size, a plan changes
     * the rounding of the transforms (not their result beyond it); the planner fixes it once
     * per device, size and path in a process, so that every handle of a size uses the same. */
    int32_t eval_radix;
    int32_t forward_radix;
    int32_t adjoint_radix;
    /* the solver kernel's form: 1 staged (the patch's optimiser vectors, object metric sums,
     * object tables and null-space map copied into shared memory as the kernel starts, taken
     * whenever they fit in 96 KB), 2 the global-memory form.  Both compute the same bits.
     * Set: 0 keeps; pinning the form leaves the planner on. */
    int32_t solver_form;
} rdxg_launch_shape;

/* The launch-shape planner, in place of the FFTW_MEASURE planning of the reference's
 * FourierTransform (image/fouriertransform.cpp:73-90, which times candidate plans once per
 * transform size and keeps the fastest): times every compiled shape of each kernel on the
 * loaded batch (reps launches each, CUDA events; the adjoint on the gradient list of a tenth
 * of the patches, the share of a solve round that takes gradients, and of 24 patches at least)
 * and keeps the fastest.  The first solve of a
 * handle does this by itself (or takes the shapes measured by an earlier handle of the same
 * geometry, device and batch size in this process); RDXG_AUTOTUNE=0 in the environment keeps
 * the default shapes.  FP64 handles have one shape.  chosen (or NULL): the shapes kept;
 * ms (or NULL): [6] ms per launch of eval (default, alternative), forward (...), adjoint (...),
 * 0 for kernels the handle's path does not use. */
int rdxg_autotune(rdxg_solver* h, int32_t reps, rdxg_launch_shape* chosen, double* ms);
/* Pins the shapes (0 in a field keeps that kernel's current shape); no measurement follows. */
int rdxg_set_launch_shape(rdxg_solver* h, const rdxg_launch_shape* shape);
int rdxg_get_launch_shape(const rdxg_solver* h, rdxg_launch_shape* shape);

/* Debug copies of device state (host buffers sized by the caller):
 * which = 0 D [P][I][N][N] complex, 1 OTF [P][I][N][N] complex, 2 gamma [P][nObj],
 *         3 image stats [P][I][3] (mean, stddev, noise), 4 object O [P][nObj][N][N] complex,
 *         5 shifts [P][I][2] int32, 6 phases of the last fused evaluation [P][I][n][n] float
 *         (fused FP32 path only), 7 the number of device allocations the handle holds
 *         (int64), 8 their bytes (int64).  Complex values are float pairs in FP32 mode and
 *         double pairs in FP64 mode. */
int rdxg_debug_copy(rdxg_solver* h, int32_t which, void* out, size_t bytes);

/* Debug writes of device state, to test error paths from the host without a device fault:
 * which = 0 the tensor-core mode expansion's status word (int32; non-zero is what a bounded
 * wait that gave up leaves behind: the next call that checks it returns RDXG_ERR_CUDA with the
 * message, and clears it).  No counterpart in the reference. */
int rdxg_debug_set(rdxg_solver* h, int32_t which, const void* in, size_t bytes);

/* ---- Once-per-job static inputs (host code, no device work) ----
 * What redux computes once per job on the master and ships in GlobalData; a caller may keep
 * using redux's own classes for these, or call these and pass the results in rdxg_static. */

/* Pupil::calculatePupilSize (src/lib/image/pupil.cpp:78-100): frequency cutoff, pupil radius
 * in pixels and the pupil grid size (pupilPixels, doubled as the reference returns it) for an
 * image of n_pixels at the given wavelength [m], telescope diameter [m] and image scale. */
int rdxg_pupil_size(int32_t n_pixels, double wavelength, double telescope_d, double arcsec_per_pixel,
                    double* frequency_cutoff, double* radius, int32_t* pupil_pixels);
/* makePupil (src/lib/image/utils.cpp:68-124) centred on pixel (n/2, n/2), then
 * Pupil::normalize (pupil.cpp:280-300): the anti-aliased annulus on an n x n grid scaled to
 * [0, 1]; area = the makePupil sum before scaling. */
int rdxg_make_pupil(int32_t n, double radius, double inner_radius, double* pupil, double* area);
/* Pupil::generateSupport (pupil.cpp:245-277): pupil_support (capacity n*n) = indices where the
 * pupil exceeds threshold, pupil_in_otf (or NULL; capacity n*n) = those indices in the N = 2n
 * OTF grid, otf_support (capacity 4 n*n) = indices of the centred N x N grid where the
 * pupil's autocorrelation exceeds threshold, area = the pupil summed over its support. */
int rdxg_pupil_support(const double* pupil, int32_t n, double threshold, int32_t* pupil_support,
                       int32_t* n_pupil_support, int32_t* pupil_in_otf, int32_t* otf_support, int32_t* n_otf_support,
                       double* area);

enum { RDXG_MODES_ZERNIKE = 0, RDXG_MODES_KL = 1 };
typedef struct {
    int32_t kind;            /* RDXG_MODES_ZERNIKE or RDXG_MODES_KL (BASIS) */
    int32_t pupil_pixels;    /* n */
    double radius;           /* pupil radius in pixels */
    double wavelength;       /* [m]: the modes are scaled by 1/wavelength (GlobalData::get) */
    double angle;            /* rotation of the basis (ModeInfo angle), radians */
    double jacobian_scale;   /* scale of the tilt Jacobian (ModeSet::measureJacobian) */
    int32_t kl_first;        /* KL_MIN_MODE: first Zernike of the KL expansion */
    int32_t kl_last;         /* KL_MAX_MODE: last Zernike of the KL expansion */
    double kl_cutoff;        /* SVD_REG: Zernike weights below this are dropped */
} rdxg_mode_params;
/* ModeSet::generate (src/lib/momfbd/modes.cpp:158-197, 348-437) with getNorms/normalize
 * (443-462, 524-535) and measureJacobian (464-512): modes [n_modes][n][n] for the Noll
 * indices mode_list (Zernike::getZernike, image/zernike.cpp:234-274; KL modes from the
 * Karhunen-Loeve expansion of the Noll covariance, zernike.cpp:82-125, 367-479, with the tilts
 * 2 and 3 kept Zernike), each with unit RMS over the pupil times 1/wavelength; atm_rms (or
 * NULL) = the square root of each mode's Kolmogorov variance at D/r0 = 1; tilt_jacobian (or
 * NULL) = [2][2] J_T_xy. */
int rdxg_make_modes(const rdxg_mode_params* params, const int32_t* mode_list, int32_t n_modes, double* modes,
                    double* atm_rms, double* tilt_jacobian);
/* Solver::init's windows (solver.cpp:113-126): apodizeInPlace (image/utils.cpp:584-614) of
 * all-ones patch_size^2 arrays with a blend of apodization (patch_size / 8 when negative)
 * and half of it. */
int rdxg_apodization_windows(int32_t patch_size, int32_t apodization, double* window, double* noise_window);

/* Host drop-in for redux's conjugate_rdx minimiser with the Solver::run stage loop
 * (conjugate_gradient.cpp:128-256, helpers.cpp:58-215, solver.cpp:425-537) driving
 * caller-supplied callbacks.  n_modes stages the enabled-mode count exactly as Solver::run;
 * df receives the number of enabled modes.  Writes x (n_free), the metric history and a
 * report.  Used for host-side validation of the device state machine. */
typedef double (*rdxg_f_fn)(const double* x, void* user);
typedef void (*rdxg_df_fn)(const double* x, int32_t method, int32_t mode_count, double* g, void* user);
typedef void (*rdxg_shift_fn)(const double* x, void* user);
int rdxg_cg_minimize(int32_t n_free, int32_t n_modes, const rdxg_solve_params* params,
                     double grad_scale, rdxg_f_fn f, rdxg_df_fn df, rdxg_shift_fn shift,
                     void* user, double* x_out, rdxg_patch_report* report, double* metrics);

#ifdef __cplusplus
}
#endif

#endif /* RDXG_H */
