/* libfit_gb300 — GB300-native (sm_103a) transfer hot path of FlowInvariantTransfer.jl.
 *
 * A thin C ABI (plain pointers and sizes) that a Julia `ccall` binds. Conventions follow the
 * reference package exactly:
 *   - spectral arrays are column-major (ns..., comp), interleaved complex: ComplexF64 when the
 *     plan's io_f64 = 1, ComplexF32 when io_f64 = 0 (src/Workspaces.jl:46-75);
 *   - wavenumbers ks[d] are FFTW-order vectors with +N/2 at the Nyquist index (src/Utils.jl:51-63);
 *   - shell edges are passed explicitly (computed by shell_edges, src/ShellBinning.jl:50-79);
 *     shell indices are Int64, 1-based, 0 = no shell (src/ShellBinning.jl:126-140);
 *   - T(n,m) is written column-major (n fastest);
 *   - every real result is FP64 (the caller converts to the input precision when it wants the
 *     reference's result element type).
 * ptr_kind: FIT_PTR_HOST (0) = all array arguments are host memory (copied in/out inside the
 * call); FIT_PTR_DEVICE (1) = all array arguments are device memory. Every call is synchronous
 * on the plan's stream and returns FIT_OK (0) or a negative error code; fit_last_error() gives
 * the message (thread-local). Plans are not re-entrant; distinct plans may be used from
 * distinct threads.
 */
#ifndef FIT_GB300_H
#define FIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FIT_OK 0
#define FIT_ERR_ARG -1
#define FIT_ERR_SIZE -2
#define FIT_ERR_CUDA -3
#define FIT_ERR_ALLOC -4
#define FIT_ERR_STATE -5

#define FIT_PTR_HOST 0
#define FIT_PTR_DEVICE 1

/* dealiasing (src/Types.jl:458-476) */
#define FIT_DEALIAS_NONE 0
#define FIT_DEALIAS_TWO_THIRDS 1
#define FIT_DEALIAS_THREE_HALVES 2

/* invariants (src/Types.jl:77-132) */
#define FIT_INV_KINETIC_ENERGY 0
#define FIT_INV_PASSIVE_SCALAR 1
#define FIT_INV_HELICITY 2
#define FIT_INV_ENSTROPHY 3

/* decompositions (src/Types.jl) */
#define FIT_DECOMP_HELICAL 1
#define FIT_DECOMP_HELMHOLTZ 2
#define FIT_DECOMP_TOROIDAL_POLOIDAL 3  /* src/Decomposition.jl:107-141 (3D) */

/* shell-to-shell execution forms */
#define FIT_S2S_PLAIN 0    /* one nonlinear term per mediator shell, launched one by one */
#define FIT_S2S_BATCHED 1  /* mediators batched, fused kernels, CUDA-graph replay */

typedef struct fit_plan fit_plan;

/* Creates a plan (device buffers, transform tables, one CUDA stream) for fields on grid
 * ns[0..nd) with n_advected components (M) advected by a velocity of n_advecting (D >= nd)
 * components. precision = 64 or 32 (arithmetic of the transforms and products; reductions are
 * always FP64). Replaces the workspace + FFTW plan construction of
 * ext/FlowInvariantTransferFFTWExt.jl:37-49 (src/Workspaces.jl:22,63-75). */
int fit_plan_create(fit_plan** out, int nd, const int64_t* ns, int n_advected, int n_advecting, int dealias,
                    int precision, int io_f64, const double* const* ks);
int fit_plan_destroy(fit_plan* plan);
const char* fit_last_error(void);
/* Use an existing cudaStream_t (passed as void*) instead of the plan's own stream. */
int fit_plan_set_stream(fit_plan* plan, void* stream);
/* info[0..8] = nd, N0, N1, N2, M0, M1, M2 (transform grid), bytes of device memory held, bytes of
 * host inputs copied to the device by the plan's calls so far. */
int fit_plan_info(const fit_plan* plan, int64_t* info, int n);
/* Number of library kernels launched since load (graph replays count their kernels). */
long long fit_launch_count(void);
/* Per-launch profiling: when enabled, every launch is bracketed by CUDA events and tagged with its
 * algorithmic DRAM bytes (captured graphs are bypassed while enabled). fit_prof_read sums one
 * kernel kind (0..13, named by fit_prof_kind_name) since the last fit_prof_enable. */
int fit_prof_enable(int on);
int fit_prof_read(int kind, double* ms_total, double* bytes_total, long long* launches);
const char* fit_prof_kind_name(int kind);

/* N̂ = FFT[(u_adv·∇) f] in the reference normalisation. Replaces
 * NonlinearTerm._compute_nonlinear_term! (src/NonlinearTerm.jl:102-116) for the FFT backend:
 * _nonlinear_term_fft! (ext/FlowInvariantTransferFFTWExt.jl:61-121) and
 * _nonlinear_term_padded_fft! (:160-183). adv_hat = NULL means self-advection. */
int fit_nonlinear_term(fit_plan* plan, const void* f_hat, const void* adv_hat, void* N_hat, int ptr_kind);

/* Shell index of every mode. Replaces shell_coordinate + assign_shells
 * (src/ShellBinning.jl:19-36,126-140). dims_mask bit d selects axis d (all bits = isotropic);
 * coord_f32 = 1 evaluates the coordinate in Float32 (Float32 wavenumbers). */
int fit_assign_shells(fit_plan* plan, const double* edges, int n_edges, uint32_t dims_mask, int coord_f32,
                      int64_t* idx_out, int ptr_kind);

/* Per-mode transfer density t(k) for an invariant. Replaces transfer_density!
 * (src/Invariants.jl:40-104). N_hat has the plan's n_advected components. */
int fit_transfer_density(fit_plan* plan, int invariant, const void* carrier, const void* N_hat, double* t_out,
                         int ptr_kind);

/* T(k_n) and Pi(K_n) = cumsum(T). Replaces calculate_spectral_flux →
 * _calculate_spectral_flux_with_N̂! (src/SpectralFlux.jl:49-94,148-180). carrier = NULL uses
 * u_hat (the decomposed-component branch passes the component as carrier, :86-91). */
int fit_spectral_flux(fit_plan* plan, const void* u_hat, const void* adv_hat, const void* carrier,
                      const double* edges, int n_edges, uint32_t dims_mask, int coord_f32, int invariant, double* T,
                      double* Pi, int ptr_kind);

/* Shell-to-shell T(n,m), net transfer and max|T+T'|. Replaces
 * ShellToShellTransfer._calculate_shell_to_shell! (src/ShellToShell/ShellToShellTransfer.jl:152-159)
 * → _shell_to_shell_fft! (ext/FlowInvariantTransferFFTWExt.jl:209-295) and the GPU/threaded
 * execution backends (ext/FlowInvariantTransferKernelAbstractionsExt.jl:68-138,
 * ext/FlowInvariantTransferOhMyThreadsExt.jl:24-97). mode = FIT_S2S_PLAIN or FIT_S2S_BATCHED.
 * max_asym receives NaN when verify = 0. Host arguments of the batched form on a 2/3 plan of a
 * fused transform size: only the 2/3-kept box of u_hat is read; page-locked host memory is read
 * by the device during the step (overlapped with its first passes), other host memory is copied
 * before it. */
int fit_shell_to_shell(fit_plan* plan, const void* u_hat, const void* adv_hat, const double* edges, int n_edges,
                       uint32_t dims_mask, int coord_f32, int invariant, int mode, int verify, double* T_colmajor,
                       double* net, double* max_asym, int ptr_kind);

/* Installs a caller's shell index as the plan's shell table: one Int64 per grid mode, column-major
 * over ns, 1-based, 0 = no shell, exactly as assign_shells returns it and as
 * ShellToShellWorkspace keeps it in ws.shell_idx (src/Workspaces.jl:154-169,
 * src/ShellBinning.jl:126-140) for whatever shell geometry the workspace was built with.
 * n_shells = length(edges) - 1. An entry outside [0, n_shells] returns FIT_ERR_ARG. The table
 * stays installed until a call that passes shell edges replaces it. */
int fit_set_shell_index(fit_plan* plan, const int64_t* shell_idx, int n_shells, int ptr_kind);

/* fit_shell_to_shell binned by the installed shell index instead of edges: the mediator loop of
 * ext/FlowInvariantTransferFFTWExt.jl:245-275 (src/ShellToShell/ShellToShellTransfer.jl:193-224),
 * which restricts and bins by ws.shell_idx. FIT_ERR_STATE when no index is installed. Repeated
 * calls with the same pointers replay the batched form's CUDA graph, as fit_shell_to_shell does. */
int fit_shell_to_shell_indexed(fit_plan* plan, const void* u_hat, const void* adv_hat, int invariant, int mode,
                               int verify, double* T_colmajor, double* net, double* max_asym, int ptr_kind);

/* Helical (Craya-Herring) split u = u+ + u- (src/Decomposition.jl:63-98). */
int fit_helical_decompose(fit_plan* plan, const void* u_hat, void* u_plus, void* u_minus, int ptr_kind);
/* Rotational/divergent split of a 2D field (spectral Leray projection; the reference delegates
 * to HelmholtzDecomposition.jl, ext/FlowInvariantTransferHelmholtzDecompositionExt.jl:50-104). */
/* ToroidalPoloidalDecomposition (src/Decomposition.jl:107-141): u_hat (ns..., 3) -> tor, pol. */
int fit_toroidal_poloidal_decompose(fit_plan* plan, const void* u_hat, void* tor, void* pol, int ptr_kind);
int fit_helmholtz_decompose(fit_plan* plan, const void* u_hat, void* u_rot, void* u_div, int ptr_kind);

/* Partial fluxes T^{sk,sp,sq}(k_n) of a two-component decomposition (8 channels). Replaces
 * calculate_partial_fluxes (src/SpectralFlux.jl:240-285); invariant = FIT_INV_HELICITY swaps the
 * density at :277. T_channels[(sk*4 + sp*2 + sq)*n_shells + n], component 0 = positive /
 * rotational, 1 = negative / divergent. */
int fit_partial_fluxes(fit_plan* plan, const void* u_hat, int decomposition, int invariant, const double* edges,
                       int n_edges, uint32_t dims_mask, int coord_f32, double* T_channels, int ptr_kind);

/* The 8 partial-flux channels of n_invariants invariants (KE, Helicity, Enstrophy codes) from one
 * pass: calculate_partial_fluxes (src/SpectralFlux.jl:240-285) for each invariant, sharing the four
 * nonlinear terms (u_sp . grad) u_sq between invariants and the component transforms between
 * terms. T_channels[(j*8 + sk*4 + sp*2 + sq)*nsh + n] for invariant j. The first call for a set of
 * pointers runs eagerly, the second captures a CUDA graph (on a plan stream other than the legacy
 * default stream), later calls replay it. */
int fit_partial_fluxes_batched(fit_plan* plan, const void* u_hat, int decomposition, const int* invariants,
                               int n_invariants, const double* edges, int n_edges, uint32_t dims_mask, int coord_f32,
                               double* T_channels, int ptr_kind);

/* Resolved S(k|p) (column-major [k..., p...]) and net(k) = sum_p S(k|p). Replaces
 * calculate_mode_to_mode_transfer (src/ScaleToScale/ScaleToScaleTransfer.jl:49-91).
 * fp64_products = 1 evaluates every triad in FP64, 0 in FP32 with FP64 sums. */
int fit_mode_to_mode(fit_plan* plan, const void* u_hat, const void* adv_hat, int invariant, int fp64_products,
                     double* S, double* net, int ptr_kind);

/* Coarse-graining energy flux Pi_ell(x) = -tau_ij S_ij of the physical velocity u = sum_k û e^{ikx}
 * (û = fft(u)/Np), filter_kind 0 sharp / 1 Gaussian / 2 top-hat at scale ell (src/Filters.jl:19-26).
 * Restates calculate_coarse_graining_flux (src/CoarseGrainingFlux.jl:60-72), which the reference
 * delegates to the 2D-only CoarseGrainingEnergyFluxes.jl, for 2D and 3D. Pi is written in the plan
 * precision (N^D points, x fastest); A_out (nd*nd fields of d_j ū_i, component i*nd+j) and tau_out
 * (nd(nd+1)/2 fields, order 00 11 22 01 02 12) are optional outputs in the plan precision;
 * Pi_mean is the mean. u_hat uses the package convention û = fft(u)/Np. */
int fit_coarse_graining_flux(fit_plan* plan, const void* u_hat, double ell, int filter_kind, void* Pi,
                             void* A_out, void* tau_out, double* Pi_mean, int ptr_kind);

/* û = fft(u)/Np (the package coefficient convention, src/FlowInvariantTransfer.jl:242) of the
 * plan's n_advected real physical fields (x fastest, io element type), written as the full N-grid
 * spectrum. Replaces the host FFTW.fft a caller of the reference runs before every spectral call;
 * unpadded plans only. */
int fit_forward_spectrum(fit_plan* plan, const void* u_phys, void* u_hat, int ptr_kind);

/* Advances û in place by nsteps of SSP-RK3 for forced incompressible Navier-Stokes,
 * dû/dt = -P[N̂(û)] - nu k^2 û + alpha û 1[0 < |k| <= kf], alpha = power / (2 E_f), with this
 * library's nonlinear term (the plan's dealiasing). The reference's examples/flows.jl:28-89
 * evolver is unforced RK2; this forced RK3 form has no reference counterpart. */
int fit_ns_evolve(fit_plan* plan, void* u_hat, int nsteps, double dt, double nu, double kf, double power,
                  int ptr_kind);

/* Smooth band-to-band transfer T(n,m) between log-Gaussian bands (partition of unity of
 * exp(-(ln(kappa/centers[n]))^2 / (2 logwidth^2)) over the shell coordinate kappa of dims_mask).
 * Replaces calculate_band_to_band_transfer (src/BandTransfer.jl:71-113): one nonlinear term per
 * band m of w_m * u_hat advected by adv_hat (NULL = u_hat), its transfer density against u_hat,
 * weighted by w_n. T_colmajor[n + nb*m] (nb*nb doubles), net[n] = sum_m T(n,m), max_asym =
 * max |T(n,m) + T(m,n)|. 1..16 bands. */
int fit_band_to_band(fit_plan* plan, const void* u_hat, const void* adv_hat, const double* centers, int n_bands,
                     double logwidth, uint32_t dims_mask, int coord_f32, int invariant, double* T_colmajor,
                     double* net, double* max_asym, int ptr_kind);

/* ---- uneven batches and the transform autotuner --------------------------------------------------
 * A batch runs many spectral-flux instances, each calculate_spectral_flux / calculate_scalar_flux
 * (src/SpectralFlux.jl:49-94,148-180,203-269) on its own plan (grid, dimension, invariant, shell
 * geometry and edges may all differ), as one CUDA graph launch. The reference computes such a set
 * one call at a time; batching has no counterpart there. Pointers are device pointers fixed when
 * the instance is added; T_dev / Pi_dev receive n_edges-1 doubles (Pi_dev may be NULL). The first
 * fit_batch_run executes eagerly (allocation, autotuning), the second captures the graph over
 * n_branches concurrent branch streams and launches it, later runs only launch it. Runs are
 * asynchronous on `stream`. */
typedef struct fit_batch fit_batch;
int fit_batch_create(fit_batch** out, int n_branches);
int fit_batch_destroy(fit_batch* batch);
int fit_batch_add_flux(fit_batch* batch, fit_plan* plan, const void* u_dev, const void* adv_dev, const double* edges,
                       int n_edges, uint32_t dims_mask, int coord_f32, int invariant, double* T_dev, double* Pi_dev);
int fit_batch_run(fit_batch* batch, void* stream);
/* Every instance launched eagerly, one after the other on `stream` (no graph): the sequential form. */
int fit_batch_run_eager(fit_batch* batch, void* stream);
/* out[0..3] = instances, state (0 new, 1 eager run done, 2 graph ready), kernels in the graph, branches */
int fit_batch_info(const fit_batch* batch, int64_t* out, int n);

/* Transform-pass autotuner (global, off by default): when on, the first launch of every pass shape
 * outside a graph capture times the candidate kernels (compile-time engine; runtime engine over
 * tile widths, elements per thread and radix orders) and keeps the fastest for later launches. */
int fit_autotune_enable(int on);
int fit_autotune_clear(void);
int fit_autotune_info(int64_t* n_entries, int64_t* n_runtime_engine, double* ms_default, double* ms_best);
/* fields[0..8] = kind (0 fwd, 1 inv strided, 2 c2r, 3 r2c), N, columns or lines, batch, element
 * bytes, engine (0 compile-time, 1 runtime), C, elements per thread, radix order; ms = best, default. */
int fit_autotune_entry(int64_t i, int64_t* fields, double* ms);

/* Benchmark hook (no counterpart in the reference): times one kernel of the fused shell-to-shell
 * pipeline alone on synthetic device data, mediators of full extent on an N^3 grid under the
 * 2/3 rule, N in {64, 128, 256, 512}; reps launches after one warm-up. pass 0: the x pass (inverse
 * x transforms, product with the advecting velocity, forward x transform) of one mediator over
 * `units` x lines (a multiple of 16, at most N^2); pass 1: the y-inverse pass of one mediator over
 * `units` z planes (at most N); pass 2: the z-forward + shell-binning pass of `units` mediators (at
 * most 8) over all pencils, 32 shells of width 14 N / 512. ms_per_launch = mean launch time,
 * alg_bytes = the launch's algorithmic bytes. Allocates its buffers for the call and frees them
 * (at N = 512: about 2.3 GB for the x pass over 65536 lines, 4.6 GB for the y pass, 1.2 GB + 0.7 GB
 * per mediator for the z pass). */
int fit_bench_fused_pass(int pass, int N, long long units, int reps, double* ms_per_launch, double* alg_bytes);

/* ---- learned subfilter-stress closure (no counterpart in the reference) -------------------------
 * A pointwise MLP 9 -> 64 -> 64 -> 6 (ReLU) maps the filtered velocity-gradient tensor A_ij = d_j ū_i
 * (9 features) to the six subfilter-stress components (tau_00 tau_11 tau_22 tau_01 tau_02 tau_12).
 * Tensor-core kernels: BF16 operands (weights, features, activations), FP32 accumulation, on the
 * fifth-generation tensor cores (tcgen05 MMAs, accumulators in tensor memory) for both the forward
 * and the training step. params is
 * the FP32 master copy (fit_mlp_nparams() floats: W1[64][16], b1[64], W2[64][64], b2[64], W3[8][64],
 * b3[8]; input columns 9..15 and output rows 6..7 are padding that stays zero). Point data is
 * field-major with field stride ld >= P: X[9][ld], T/Y[6][ld]. Features are multiplied by
 * in_scale[9] and targets by t_scale[6] before the network sees them; fit_mlp_forward divides its
 * outputs by t_scale again. homogeneous != 0: with v the scaled features and s = |v|^2, the network
 * sees v/|v| and its outputs are multiplied by s (a stress homogeneous of degree 2 in A). All
 * pointers are device pointers; stream may be NULL. */
int fit_mlp_nparams(void);
/* Y (6 x ld, optional) = predicted stress; Pi (P, optional) = -tau_ij S_ij of the prediction with
 * S = (A + A^T)/2 taken from the unscaled features (the closure's flux, fused). clark_ell > 0: the
 * network is a residual over the gradient model and ell^2/12 A A^T is added to its output. */
int fit_mlp_forward(const float* params, const float* X, int64_t ld, int64_t P, const float* in_scale,
                    const float* t_scale, int homogeneous, double clark_ell, float* Y, float* Pi, void* stream);
/* *timed_out = 1 when a clock-bounded wait of an earlier fit_mlp_forward or fit_mlp_train_grad gave
 * up (its outputs are then not valid); reading synchronises the device and clears the flag. */
int fit_mlp_status(int* timed_out);
/* out (6 x ld) = tau - ell^2/12 A A^T: residual targets of a network trained over the gradient model. */
int fit_stress_residual(const float* A, const float* tau, int64_t ld, int64_t P, double ell, float* out,
                        void* stream);
/* Adds to grad (not cleared) the gradient of loss = sum_p sum_o (s_p y_po - t_scale_o T_op)^2 / Ptot
 * (y: network output, s_p = 1 unless homogeneous) over the P points given (Ptot: points of the
 * whole minibatch, for split calls), and to *loss the sum of squared scaled errors. */
int fit_mlp_train_grad(const float* params, const float* X, const float* T, int64_t ld, int64_t P, int64_t Ptot,
                       const float* in_scale, const float* t_scale, int homogeneous, float* grad, double* loss,
                       void* stream);
/* One Adam step (bias-corrected, step >= 1) on params with moment buffers m, v. */
int fit_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                 float beta2, float eps, void* stream);

/* Gradient (Clark) model baseline for a Gaussian filter, tau_ij = ell^2/12 A_ik A_jk, on the same
 * field-major A (9 x ld): tau (6 x ld) and/or Pi = -tau_ij S_ij (P), each optional. */
int fit_gradient_model_flux(const float* A, int64_t ld, int64_t P, double ell, float* tau, float* Pi,
                            void* stream);
/* FP64 reductions for normalisation and scoring, device outputs: fit_field_moments writes
 * (sum x, sum x^2) per field (2*nf doubles); fit_field_compare writes (sum a, sum b, sum a^2,
 * sum b^2, sum ab, sum (a-b)^2). */
int fit_field_moments(const float* X, int64_t ld, int64_t P, int nf, double* out, void* stream);
int fit_field_compare(const float* a, const float* b, int64_t P, double* out, void* stream);

/* Allocation-free variant of fit_mode_to_mode, for callers that cannot allocate device memory
 * (a caller-owned memory budget or allocator, a latency-critical loop where an allocation would
 * synchronise the device, an embedding runtime that only lends its own buffers). It has no
 * counterpart in the reference. Every array argument is a device pointer (ks_dev: nd device
 * arrays); no plan is used and nothing is allocated: intermediates live in one fixed 6.5 MiB
 * device array that each GPU loading the library holds until exit. Grids of at most 32768 modes
 * (32^3); larger grids return FIT_ERR_SIZE. Every array argument (ks_dev[d] included) must be
 * device or managed memory: NULL tables and host pointers return FIT_ERR_ARG before anything is
 * launched. The first call on a device looks up that array's device address (do it before any
 * stream capture); the address is kept for the process, so the entry point must not be used again
 * after cudaDeviceReset. Calls share the array, so calls that overlap on the GPU race: serialise
 * them per device. The call synchronises `stream` before returning, except while that stream is
 * being captured (it then returns once the work is enqueued). stream may be NULL (default
 * stream). */
int fit_mode_to_mode_noalloc(int nd, const int64_t* ns, int n_advected, int n_advecting, int dealias,
                             const double* const* ks_dev, int invariant, int fp64_products, int io_f64,
                             const void* u_hat, const void* adv_hat, double* S, double* net, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FIT_GB300_H */
