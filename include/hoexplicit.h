/*
 * hoexplicit.h — C ABI of libhoexplicit.so, the GB300 (sm_103a) explicit
 * higher-order MRI encoding operator.
 *
 * The operator is
 *
 *   y[s,c] = (1/sqrt(nVox)) * sum_{v in mask} exp(+i*2*pi*phi[s,v]) * x[v] * csm[v,c]
 *   phi[s,v] = sum_l bf[v,l] * kspha[l,s] + times[s] * fieldmap[v]      (cycles)
 *
 * with the adjoint writing zeros outside the mask.  Units follow the
 * reference: coefficients in cycles/m^p, coordinates in metres, times in
 * seconds, fieldmap in Hz.  Layouts follow the reference's Julia arrays
 * (column-major):
 *   image x   : complex64 [prod(matrixSize)], x index fastest
 *   data  y   : complex64 [nSam*nCha], samples fastest, then coils
 *   bf        : float64 [nVox x nTermEff]      element (v,l) at v + l*nVox
 *   kspha     : float64 [nTermEff x nSam]      element (l,s) at l + s*nTermEff
 *   csm       : complex128 [nVox x nCha]       element (v,c) at 2*(v + c*nVox)
 *
 * Reference interfaces each entry point replaces (paths inside the
 * HighOrderMRI.jl tree):
 *   hoe_create        ExplicitGPUOp constructor,
 *                     src/EncodingOperator/Explicit/explicit_gpu_operator.jl:299-392
 *                     (model preparation by prep_kspha / basisfunc_spha /
 *                     prep_concomitant stays on the caller's side, as in
 *                     array_operator.jl:124-139)
 *   hoe_forward       explicit_gpu_forward!, explicit_gpu_operator.jl:226-246
 *                     (math of explicit_array_forward, array_operator.jl:241-288)
 *   hoe_adjoint       explicit_gpu_adjoint!, explicit_gpu_operator.jl:248-270
 *                     (math of explicit_array_adjoint, array_operator.jl:294-348)
 *   hoe_normal        explicit_gpu_normal!, explicit_gpu_operator.jl:272-297, with the
 *                     weight checks of normalOperator, explicit_gpu_operator.jl:399-416
 *   hoe_derivative    explicit_array_derivative, array_operator.jl:187-235
 *                     (the kspha_dt mode used by FindDelay, FindDelay.jl:195-200)
 *   hoe_backward      no reference counterpart: gradient of 0.5*||E x - y||^2 with
 *                     respect to kspha, fieldmap and a time origin t0
 *   hoe_recon         recon_HOOp, src/Recon/recon_HOOp.jl:52-88, for the resident
 *                     explicit operator: the weighting W∘HOOp and normal EᴴWᴴWE of
 *                     :73-78 and the CGNR solve!(solver, Data) of :79-80
 *                     (RegularizedLeastSquares CGNR with L2Regularization)
 *   hoe_batch_*       no batched counterpart: the reference builds one operator per
 *                     slice (explicit_gpu_operator.jl:299-392) and calls its products
 *                     and recon_HOOp (recon_HOOp.jl:52-88) slice by slice; a batch
 *                     runs all slices' products in one persistent launch per
 *                     direction and their CGNR solves in one CUDA graph
 *   hoe_set_kspha     the per-iteration operator rebuilds of FindDelay.jl:190-193
 *                     (HighOrderExplicitOp(gridding, kspha_τ, datatime; ...)), done on
 *                     the device for the sample side only
 *   hoe_kdot_stencil  kspha_dt of FindDelay.jl:179-180
 *   hoe_interp_traj_time
 *                     InterpTrajTime, src/Synchronization/InterpTraj.jl:18-40 (Akima)
 *   hoe_find_delay    FindDelay, src/Synchronization/FindDelay.jl:139-214
 *   hoe_find_delay_multishot
 *                     FindDelay_multishot, src/Synchronization/FindDelay_multishot.jl:65-158
 *   hoe_coil_gram / hoe_coil_fit / hoe_coil_apply
 *                     estimate_noise_covariance, fit_coil_compression and
 *                     apply_coil_compression, src/Recon/CoilCompression.jl:127-301
 *   hoe_sfu_rate      no reference counterpart (calibration of the roofline ceiling)
 *   hoe_autotune      no reference counterpart (the reference's backend and nBlock
 *                     are chosen by the caller, HighOrderExplicitOp.jl:48-50)
 *   hoe_close         Base.close(::ExplicitGPUOp), explicit_gpu_operator.jl:435-446
 *   hoe_free          releases the host handle (Julia finalizer)
 *   hoe_set_timing / hoe_get_timings
 *                     CUDA-event tracing; replaces the reference's ad-hoc @elapsed
 *                     timing of the legacy path, kernel_operator.jl:333-349
 *
 * Conventions: every entry point returns HOE_OK (0) or a negative HOE_ERR_*
 * code; nothing throws across the ABI.  The message of the last failure is
 * kept per handle (hoe_last_error) or per thread for failures without a
 * handle (hoe_last_error(NULL)).  Device pointers are caller-owned, on the
 * handle's device, and are never freed by the library.  Calls are ordered on
 * the stream argument (a cudaStream_t; NULL = legacy default stream).  A handle
 * owns scratch space and is not reentrant: one call at a time per handle.
 */
#ifndef HOEXPLICIT_H
#define HOEXPLICIT_H

#include <stdint.h>

#if defined(__GNUC__)
#define HOE_API __attribute__((visibility("default")))
#else
#define HOE_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define HOE_ABI_VERSION 2

/* status codes */
#define HOE_OK               0
#define HOE_ERR_ARG         -1   /* invalid argument (Julia ArgumentError)        */
#define HOE_ERR_DIM         -2   /* inconsistent sizes (Julia DimensionMismatch)  */
#define HOE_ERR_OOM         -3   /* device allocation failed (OutOfMemoryError)   */
#define HOE_ERR_CUDA        -4   /* CUDA runtime error                            */
#define HOE_ERR_TIMEOUT     -5   /* a bounded device wait ran out                 */
#define HOE_ERR_CLOSED      -6   /* handle was closed (Julia ArgumentError)       */
#define HOE_ERR_UNSUPPORTED -7   /* mode not available on this device/build       */

/* contraction engines (hoe_desc.engine, hoe_set_engine) */
#define HOE_ENGINE_FP32_SIMT  0  /* plain FP32 CUDA-core direct kernel              */
#define HOE_ENGINE_TC_BF16X3  1  /* tcgen05 tensor cores, split-BF16 3-product, FP32 accumulate */
#define HOE_ENGINE_AUTO       2  /* hoe_create / hoe_set_engine: the tensor-core engine where the device
                                    (sm_103), the coil count (<= 64) and the plan's residual phase bound
                                    (<= 1024 cycles, hoe_info.residual_phase_bound) allow it, else FP32;
                                    hoe_get_info reports the choice */

/* hoe_backward flags */
#define HOE_GRAD_KSPHA     1     /* write dL/dkspha                                   */
#define HOE_GRAD_FIELDMAP  2     /* write dL/dfieldmap                                */
#define HOE_GRAD_T0_B0     4     /* dL/dt0 includes the fieldmap part  -fieldmap[v]   */
#define HOE_GRAD_T0_COEF   8     /* dL/dt0 includes the coefficient part -bf.kspha_dt */

typedef struct hoe_handle hoe_handle;
typedef struct hoe_batch hoe_batch;

typedef struct hoe_desc {
    int32_t abi_version;      /* = HOE_ABI_VERSION                                     */
    int32_t nX, nY, nZ;       /* grid matrix size                                      */
    int32_t nSam;             /* samples                                               */
    int32_t nCha;             /* coils                                                 */
    int32_t nTerm;            /* spherical-harmonic terms: 9 or 16                     */
    int32_t has_concomitant;  /* 1: bf/kspha carry 4 appended concomitant terms        */
    int32_t nVox;             /* masked voxels (count(mask)) > 0                        */
    int32_t engine;           /* HOE_ENGINE_*                                          */
    int32_t device;           /* CUDA device ordinal; -1 = current device              */
    int32_t tc_plan;          /* tensor-core execution plan: 0 = default; 1-4 (up to 16
                                 coils): the variants hoe_autotune times (hoe_tune_result) */
    int32_t reserved;         /* must be 0                                             */
    int32_t split_hint;       /* 0 = automatic split-K                                 */
    const int32_t *mask_idx;  /* host [nVox], 0-based linear grid indices, ascending   */
    const double  *bf;        /* host [nVox x nTermEff], nTermEff = nTerm + 4*has_conc */
    const double  *kspha;     /* host [nTermEff x nSam], prepared (prep_kspha applied) */
    const double  *times;     /* host [nSam] seconds                                   */
    const double  *fieldmap;  /* host [nVox] Hz, masked; NULL = zeros                  */
    const double  *csm;       /* host complex [nVox x nCha], masked; NULL = ones (nCha must be 1) */
    const double  *kspha_dt;  /* host [nTerm x nSam] or NULL: dkspha/dt (derivative & t0 gradient) */
} hoe_desc;

typedef struct hoe_timings {
    float   forward_kernel_ms;     /* main contraction kernel of the last forward   */
    float   adjoint_kernel_ms;     /* main contraction kernel of the last adjoint   */
    float   forward_total_ms;      /* whole last forward (prologue..epilogue)       */
    float   adjoint_total_ms;      /* whole last adjoint                            */
    int64_t launches;              /* kernels launched by this handle so far        */
} hoe_timings;

/* Parameters of hoe_recon (the recParams of recon_HOOp). */
typedef struct hoe_cg_params {
    int32_t iterations;            /* maximum CG iterations (:iterations), >= 0          */
    int32_t use_graph;             /* nonzero: run the solve as one cached CUDA graph    */
    double  rel_tol;               /* stop once ||z_k|| <= rel_tol*||z_0|| (:relTol)     */
    double  lambda;                /* L2Regularization weight, >= 0 (:reg)               */
} hoe_cg_params;

/* Solver state after hoe_recon (filled when a stats pointer is given). */
typedef struct hoe_cg_stats {
    int32_t iterations;            /* iterations that updated x                          */
    int32_t status;                /* 0 iteration limit, 1 converged (rel_tol),
                                      2 stopped: p^H(E^H E + lambda I)p <= 0 or not finite */
    double  residual0;             /* ||z_0|| = ||E^H W^H W data||                        */
    double  residual;              /* ||z_k|| = ||E^H W^H (W data - W E x) - lambda x||   */
} hoe_cg_stats;

/* Parameters of hoe_find_delay (the keywords of FindDelay). */
typedef struct hoe_delay_params {
    double  start_time;            /* StartTime (s): coefficient sample j sits at
                                      (j-1)*dt - (start_time + tau)                      */
    double  dt;                    /* coefficient sampling interval (s), > 0             */
    double  dtau_min;              /* Δτ_min (s), > 0: stop once |Δτ| <= dtau_min        */
    double  jump_fact;             /* JumpFact, >= 1 (reference default 3)               */
    double  lambda;                /* L2Regularization weight of the image solve, >= 0   */
    const double *term_mask;       /* HOST [nTerm] factors from recon_terms, or NULL     */
    int32_t iter_max;              /* CGNR iterations per image solve (default 10)       */
    int32_t max_outer;             /* bound on delay updates (the reference has none)    */
} hoe_delay_params;

typedef struct hoe_delay_result {
    double  tau;                   /* returned delay tau_last - dtau/J*(J-1) (s)         */
    double  tau_last;              /* accumulated delay (s)                              */
    double  dtau;                  /* last increment (s)                                 */
    double  jump;                  /* final JumpFact                                     */
    int32_t iterations;            /* delay updates made                                 */
    int32_t status;                /* 0 converged, 1 max_outer reached,
                                      2 stopped: ||B x|| = 0 or a non-finite update      */
} hoe_delay_result;

/* Result of hoe_autotune: the candidates tried, in order, and the choice. */
typedef struct hoe_tune_result {
    int32_t engine;                /* chosen engine                                       */
    int32_t split_forward;         /* chosen split-K factors of the FP32 engine           */
    int32_t split_adjoint;
    int32_t candidates;            /* entries used below (<= 8)                           */
    int32_t cand_engine[8];
    int32_t cand_split[8];         /* forward split-K factor (FP32 engine), 0 otherwise   */
    float   cand_ms[8];            /* mean forward+adjoint time of each candidate (ms)    */
    int32_t tc_plan;               /* chosen tensor-core plan (kept if the FP32 engine wins) */
    int32_t cand_plan[8];          /* tensor-core plan of each candidate, -1 for FP32     */
} hoe_tune_result;

typedef struct hoe_batch_info {
    int32_t n;                     /* member operators                                   */
    int32_t contraction_launches;  /* contraction kernels per direction for all members  */
    int64_t launches;              /* kernels launched by batch calls so far             */
} hoe_batch_info;

typedef struct hoe_info {
    int32_t nSam, nCha, nVox, nTermEff, nFull;
    int32_t engine;
    int32_t tile_samples, tile_voxels;
    int32_t n_sample_tiles, n_voxel_tiles;
    int32_t split_forward, split_adjoint;
    int32_t residual_rank;         /* dimension r of the reduced residual phase basis */
    int32_t residual_width;        /* stored width (r rounded up to 8, 12, 16 or 24)  */
    double  residual_phase_bound;  /* max |sum_l dbeta*kappa| in cycles over all tiles */
    int64_t device_bytes;          /* device memory owned by the handle */
    int32_t tc_plan;               /* execution plan of the tensor-core contraction    */
    int32_t tc_plans;              /* plans available: 5 up to 16 coils, else 1        */
} hoe_info;

/* Library */
HOE_API const char *hoe_version(void);
HOE_API int  hoe_abi_version(void);

/* Handle lifetime */
HOE_API int  hoe_create(hoe_handle **out, const hoe_desc *desc);
/* Validates a descriptor and reports the operator's host-side plan (tiles,
 * residual rank/width, residual phase bound) without touching any device. */
HOE_API int  hoe_plan(const hoe_desc *desc, hoe_info *out);
HOE_API int  hoe_close(hoe_handle *h);     /* idempotent; later calls return HOE_ERR_CLOSED */
HOE_API void hoe_free(hoe_handle *h);      /* closes if needed and frees the host object   */
HOE_API int  hoe_is_closed(const hoe_handle *h);
HOE_API const char *hoe_last_error(const hoe_handle *h);
HOE_API int  hoe_get_info(const hoe_handle *h, hoe_info *out);
HOE_API int  hoe_set_engine(hoe_handle *h, int32_t engine);
/* Tracing: with timing enabled, CUDA events are recorded on the call's stream
 * around each forward/adjoint and its main kernel; hoe_get_timings waits for
 * the last recorded events and reports their durations and the launch count. */
HOE_API int  hoe_set_timing(hoe_handle *h, int32_t enable);
HOE_API int  hoe_get_timings(hoe_handle *h, hoe_timings *out);
/* Waits for the stream and reports a device-side failure of an earlier call:
 * HOE_ERR_TIMEOUT when a bounded wait inside a kernel ran out (the kernel
 * then skipped its remaining work).  The word is cleared after reporting. */
HOE_API int  hoe_check(hoe_handle *h, void *stream);

/* Times forward+adjoint of this operator for each available execution plan
 * with CUDA events on `stream`, `reps` repetitions each, and keeps the
 * fastest: the FP32 engine at split-K factors 1/4, 1/2 and 1 of its default,
 * and the tensor-core engine's plans.  Up to 16 coils there are five: the
 * default (3 groups of 4 phase warps, the deepest stage ring that fits,
 * accumulators flushed every 32 stages), 2 or 4 phase-warp groups, a stage
 * ring of 4, and a flush every 16 stages; above 16 coils the default only.
 * The chosen tensor-core plan serves the operator's forward, adjoint and
 * normal products (batches and the derivative product use plan 0).  Waits
 * for the stream.  Counterpart of choosing :array / :kernel / nBlock
 * (explicit_gpu_operator.jl:333, array_operator.jl:129-135) by hand. */
HOE_API int  hoe_autotune(hoe_handle *h, int32_t reps, hoe_tune_result *out, void *stream);

/* Operator applications (complex64 device vectors) */
HOE_API int  hoe_forward(hoe_handle *h, const void *x_dev, void *y_dev, void *stream);
HOE_API int  hoe_adjoint(hoe_handle *h, const void *y_dev, void *x_dev, void *stream);
/* D_dev: float [nSam*nCha] real >= 0 (W^H W, samples fastest) or NULL for ones.
 * Weight validation (finite, non-negative, real) is done by the host caller,
 * as in normalOperator; the device diagonal is used as given. */
HOE_API int  hoe_normal(hoe_handle *h, const float *D_dev, const void *x_dev, void *out_dev, void *stream);
/* B x of the kspha_dt mode: requires desc.kspha_dt (or hoe_set_kspha with
 * kspha_dt).  The tensor-core engine forms it, up to 16 coils, in one pass of
 * the forward contraction whose phase tile is scaled by 2 pi i F with
 * F = sum_l kdot_l bf_l; above 16 coils from ceil(nTerm / (64 / padded
 * coils)) forward passes of virtual coils.  The FP32 engine uses one fused
 * kernel.  The first call allocates the engine's derivative buffers. */
HOE_API int  hoe_derivative(hoe_handle *h, const void *x_dev, void *y_dev, void *stream);
/* Gradient of L = 0.5*||E x - y||^2 given the residual r = E x - y.
 *   dk_dev   float [nTermEff x nSam] (same layout as kspha) or NULL
 *   ddf_dev  float [prod(matrixSize)], zero outside the mask, or NULL
 *   dt0_dev  double [1] or NULL
 * flags: HOE_GRAD_* bits.  Coverage: the tensor-core engine up to 32 coils
 * (residual width <= 16 above 16 coils), the FP32 engine up to 16 coils;
 * beyond that HOE_ERR_UNSUPPORTED. */
HOE_API int  hoe_backward(hoe_handle *h, const void *x_dev, const void *r_dev,
                  float *dk_dev, float *ddf_dev, double *dt0_dev,
                  int32_t flags, void *stream);

/* Weighted reconstruction, recon_HOOp for this operator:
 *   x = argmin ||W (E x - data)||^2 + lambda ||x||^2   by CGNR from x = 0,
 * with W = diag(weights) repeated over the coils.
 *   data_dev     complex64 [nSam*nCha], samples fastest (Data of recon_HOOp)
 *   weights_dev  complex64 [nSam] raw sample weights (NULL: ones); a weight
 *                contributes |w|^2 to the normal, as in recon_HOOp
 *   x_dev        complex64 [prod(matrixSize)] output image, x fastest
 * All vectors and scalars stay on the device; the call is stream-ordered and
 * does not wait unless stats is non-NULL (then it waits for the stream and
 * reports the solver state).  With use_graph the iterations are captured once
 * into a CUDA graph that is cached on the handle and replayed while the
 * pointers, parameters and engine stay the same.  Results are deterministic
 * and identical with and without the graph. */
HOE_API int  hoe_recon(hoe_handle *h, const void *data_dev, const void *weights_dev, void *x_dev,
                       const hoe_cg_params *params, hoe_cg_stats *stats, void *stream);

/* Trajectory preprocessing (no handle).  traj_dev: float64 [nField x nTerm]
 * column-major (the reference's (nFieldSample, nTerm) coefficient series). */
HOE_API int  hoe_kdot_stencil(const double *traj_dev, int64_t nField, int32_t nTerm, double dt,
                              double *out_dev, void *stream);
/* InterpTrajTime: Akima interpolation of every column at datatime_dev
 * [nData], coefficient sample j at j*dt - delTime (0-based), zero outside.
 * layout 0: out [nData x nTerm] column-major (the reference's result);
 * layout 1: out [nTerm x nData] column-major (the operator's kspha layout). */
HOE_API int  hoe_interp_traj_time(const double *traj_dev, int64_t nField, int32_t nTerm, double dt,
                                  double delTime, const double *datatime_dev, int64_t nData,
                                  double *out_dev, int32_t layout, void *stream);
/* Calibration (no handle): the sin/cos rate of the special-function unit of
 * the current device in lane operations per clock per SM (sin and cos
 * counted separately), measured by a kernel that keeps every SM's unit busy
 * and reads clock64.  It allocates a few KB on `stream` and synchronises it.
 * The phase generator's ceiling is 2 operations per (voxel, sample) pair at
 * this rate. */
HOE_API int  hoe_sfu_rate(double *lanes_per_clock_per_sm, void *stream);
/* Replaces the operator's coefficients on the device: kspha_dev float64
 * [nTermEff x nSam] as desc.kspha (after prep_kspha / prep_concomitant),
 * kspha_dt_dev float64 [nTerm x nSam] or NULL (keeps the derivative table).
 * The voxel side and the reduced residual basis are kept; the sample-tile
 * anchors, residual vectors, TF32 tables and anchor-phase tables are rebuilt
 * by kernels on `stream` (no host synchronisation). */
HOE_API int  hoe_set_kspha(hoe_handle *h, const double *kspha_dev, const double *kspha_dt_dev, void *stream);
/* FindDelay on the device for an operator built on the ADC times without
 * concomitant terms: every outer iteration (coefficients and k̇ interpolated
 * at the current delay, sample-side re-plan, weighted CGNR image, y1 = data -
 * E x, y2 = B x, Δτ = J*Re(y2 \ y1)) runs as one CUDA graph; the host reads
 * a few scalars between iterations.  Density weights are the fixed
 * weights_dev (complex64 [nSam] or NULL).  x_dev (complex64 [nFull] or NULL)
 * receives the last image.  The operator keeps the last coefficients. */
HOE_API int  hoe_find_delay(hoe_handle *h, const hoe_delay_params *params, const void *data_dev,
                            const void *weights_dev, const double *traj_dev, int64_t nField,
                            void *x_dev, hoe_delay_result *out, void *stream);
/* FindDelay_multishot (src/Synchronization/FindDelay_multishot.jl:65-158): one
 * delay shared by nShot shots of a 2-D image, on the device like hoe_find_delay.
 * h is built on all nShot*nSPI samples, shot-major (sample j of shot s at
 * s*nSPI + j, the reference's reshape of (nSPI, nShot)), with the
 * concatenated ADC times.  traj_dev: each shot's coefficient series, float64
 * [nField x nTerm] column-major, shots consecutive (the reference's
 * kspha[s, :, :]); start_times: HOST float64 [nShot], the per-shot StartTime
 * (params->start_time is not used).  Shot s is interpolated at its own ADC
 * times and delay start_times[s] + tau, with its own k-dot stencil.  The image
 * update (weighted CGNR) uses h.  The residual y1 = data - E x and y2 = B x use
 * h_resid, or h when NULL: the reference builds its per-shot operators on the
 * concatenated time vector, so each shot gets the first shot's ADC times; to
 * reproduce that when the shots' times differ and the fieldmap is not zero,
 * pass an operator with the same model on the first shot's times repeated.
 * Both operators are re-planned every iteration and keep the last
 * coefficients. */
HOE_API int  hoe_find_delay_multishot(hoe_handle *h, hoe_handle *h_resid, const hoe_delay_params *params,
                                      int32_t nShot, const double *start_times, const void *data_dev,
                                      const void *weights_dev, const double *traj_dev, int64_t nField,
                                      void *x_dev, hoe_delay_result *out, void *stream);

/* SVD coil compression (src/Recon/CoilCompression.jl:150-353).  Matrices are
 * column-major: A [nObs x nCoil] observations by coils on the device
 * (complex64, or complex128 when complex128 != 0), host outputs complex128.
 *   hoe_coil_gram   G = (A - 1 m^T)^H (A - 1 m^T) in FP64 (m the column means
 *                   when center, else 0): estimate_noise_covariance divides
 *                   by nObs - 1 (center) or nObs
 *   hoe_coil_fit    fit_coil_compression: exactly one of n_virtual (> 0) and
 *                   energy_threshold (in (0, 1]); noise_cov NULL or a host
 *                   complex128 [nCoil x nCoil] covariance, scale the
 *                   prewhitening scale factor.  matrix receives W*V[:, 1:rank]
 *                   (room for nCoil x nCoil), sv the min(nObs, nCoil)
 *                   singular values of A*W
 *   hoe_coil_apply  apply_coil_compression: out [n x nVirt] = a [n x nCoil] * M
 *                   (device complex64) */
HOE_API int  hoe_coil_gram(const void *A_dev, int32_t complex128, int64_t nObs, int32_t nCoil, int32_t center,
                           double *G_host, void *stream);
HOE_API int  hoe_coil_fit(const void *A_dev, int32_t complex128, int64_t nObs, int32_t nCoil, int32_t n_virtual,
                          double energy_threshold, const double *noise_cov_host, double scale,
                          double *matrix_host, double *sv_host, int32_t *rank, double *retained_energy,
                          void *stream);
HOE_API int  hoe_coil_apply(const void *a_dev, int64_t n, int32_t nCoil, const void *M_dev, int32_t nVirt,
                            void *out_dev, void *stream);

/* Batches of operators on one device (e.g. the slices of a multi-slice scan).
 * A batch borrows its members: free the batch before freeing a member, and a
 * closed member makes every batch call return HOE_ERR_CLOSED.  When every
 * member uses the tensor-core engine and all have the same coil count, each
 * direction of all members runs in one persistent contraction launch (one per
 * residual width, at most 32 members per launch); otherwise the members are
 * applied one after another.  Vector arguments are HOST arrays of n device
 * pointers, one per member, in member order. */
HOE_API int  hoe_batch_create(hoe_batch **out, hoe_handle *const *ops, int32_t n);
HOE_API void hoe_batch_free(hoe_batch *b);
HOE_API const char *hoe_batch_last_error(const hoe_batch *b);
HOE_API int  hoe_batch_get_info(const hoe_batch *b, hoe_batch_info *out);
HOE_API int  hoe_batch_forward(hoe_batch *b, const void *const *x_dev, void *const *y_dev, void *stream);
HOE_API int  hoe_batch_adjoint(hoe_batch *b, const void *const *y_dev, void *const *x_dev, void *stream);
/* D_dev may be NULL (ones for every member) or hold NULL entries. */
HOE_API int  hoe_batch_normal(hoe_batch *b, const float *const *D_dev, const void *const *x_dev,
                              void *const *out_dev, void *stream);
/* hoe_recon for every member with the same parameters, in lockstep; weights_dev
 * may be NULL or hold NULL entries (ones); stats: NULL or n entries. */
HOE_API int  hoe_batch_recon(hoe_batch *b, const void *const *data_dev, const void *const *weights_dev,
                             void *const *x_dev, const hoe_cg_params *params, hoe_cg_stats *stats,
                             void *stream);
/* hoe_check for the batch's launches and for every member. */
HOE_API int  hoe_batch_check(hoe_batch *b, void *stream);

/* ---------------------------------------------------------------------------
 * Allocation-free forward.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory: code where cudaMalloc is
 * forbidden or unavailable, such as a reconstruction pipeline that
 * pre-allocates everything up front, or a host framework that owns every
 * device byte through its own pool.  Those callers cannot use hoe_create,
 * which allocates.  hoe_forward_noalloc computes y = E x (same result
 * convention and the plain FP32 arithmetic of hoe_forward) from a model
 * the caller already holds in device memory, and allocates nothing: no
 * cudaMalloc, no cudaFree, no allocating library call.
 *
 * Its scratch, the split-K partial sums, is one static device array of
 * 2^21 complex64 values (16 MiB).  It exists on every GPU where this
 * library's device code is loaded and stays there until the process exits.
 * Sizes are limited by it: ceil(nSam/128)*128 * nChaPad must not exceed
 * 2^21, where nChaPad is nCha rounded up to 4, 8 or a multiple of 16 (for
 * example nSam*nCha <= 2,097,152 when nCha is a multiple of 16).  Larger
 * problems are rejected with HOE_ERR_DIM and a message in
 * hoe_last_error(NULL).  nTermEff is at most 20.
 *
 * The first call on a device, with that device current, looks up the
 * scratch's device address (cudaGetSymbolAddress) and sets the kernels'
 * shared-memory limit.  Under lazy module loading (the CUDA default) that
 * first call is also when the CUDA runtime loads this library's device
 * code onto the device and allocates the 16 MiB static array, so a caller
 * that must not allocate later should make the first call during its own
 * set-up, and before any stream capture.  The address is looked up once per
 * device and not refreshed: do not call this entry point again after
 * cudaDeviceReset in the same process.
 * All calls share the one scratch array, and each call overwrites every
 * slot it reads, so nothing has to be cleared between calls.  Calls whose
 * work overlaps on the GPU (other streams, other threads) race on the
 * scratch: serialise them.
 *
 * Arrays (device, caller-owned, reference layout):
 *   mask_idx int32 [nVox]                  0-based linear grid indices of the mask
 *   bf       float64 [nVox x nTermEff]     element (v,l) at v + l*nVox
 *   kspha    float64 [nTermEff x nSam]     element (l,s) at l + s*nTermEff
 *   times    float64 [nSam]
 *   fieldmap float64 [nVox] or NULL
 *   csm      complex64 [nVox x nCha]       element (v,c) at v + c*nVox
 *   x        complex64 [nFull], y complex64 [nSam*nCha] (samples fastest)
 * ------------------------------------------------------------------------- */
typedef struct hoe_raw_model {
    int32_t nVox, nSam, nCha, nTermEff;
    const int32_t *mask_idx;
    const double  *bf;
    const double  *kspha;
    const double  *times;
    const double  *fieldmap;
    const void    *csm;
} hoe_raw_model;

HOE_API int  hoe_forward_noalloc(const hoe_raw_model *m, const void *x_dev, void *y_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* HOEXPLICIT_H */
