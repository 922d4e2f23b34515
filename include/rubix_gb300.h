/*
 * rubix_gb300 C ABI: the particle -> IFU datacube path of rubix as hand-written
 * sm_103a CUDA kernels.
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer unless its comment says "host".
 *   - All work is enqueued on `stream` (a cudaStream_t passed as void*); no call
 *     synchronises the stream and no call allocates or frees device memory.
 *     Functions that need scratch memory take a caller-provided `workspace`
 *     whose size comes from the matching *_workspace_size() query.
 *   - Return value: RUBIX_OK (0) or a negative RUBIX_E_* code; the message of the
 *     last failing call on the calling host thread is returned by
 *     rubix_last_error().  No function aborts or exits the process.
 *   - float32 data, int32 indices, row-major layouts.  A datacube is
 *     [n_spaxels][spaxel_stride] floats whose first n_wave entries of each row
 *     are the spectrum of spaxel (iy, ix) = (s / nb, s % nb) -- rubix's
 *     cube[y, x, lambda] after reshape (rubix/spectra/ifu.py:286-287).
 *
 * Each entry point names the rubix function(s) it replaces (path:line relative
 * to the rubix project root).
 */
#ifndef RUBIX_GB300_H
#define RUBIX_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define RUBIX_API __attribute__((visibility("default")))
#else
#define RUBIX_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define RUBIX_OK 0
#define RUBIX_E_INVALID (-1)     /* null pointer, negative size, bad enum      */
#define RUBIX_E_SHAPE (-2)       /* sizes inconsistent or beyond a kernel limit */
#define RUBIX_E_WORKSPACE (-3)   /* workspace missing or too small              */
#define RUBIX_E_CUDA (-4)        /* CUDA runtime or launch error                */
#define RUBIX_E_DEVICE (-5)      /* a kernel raised its device error flag       */
#define RUBIX_E_UNSUPPORTED (-6) /* valid request outside what is built        */

#define RUBIX_ABI_VERSION 1

/* Version of this ABI (RUBIX_ABI_VERSION). */
RUBIX_API int rubix_abi_version(void);

/* Message of the last failing call on this host thread ("" if none). */
RUBIX_API const char* rubix_last_error(void);

/* ------------------------------------------------------------------------- */
/* (a) Spaxel assignment and stable sort by spaxel                           */
/* ------------------------------------------------------------------------- */

/*
 * mask_out[i] = 1 if min(edges) <= x_i <= max(edges) and likewise for y_i,
 * else 0.  coords is [n][coord_stride] with x at column 0 and y at column 1.
 * Replaces mask_particles_outside_aperture, rubix/telescope/utils.py:156-178
 * (used by filter_particles, rubix/core/telescope.py:151-175).
 */
RUBIX_API int rubix_aperture_mask(const float* coords, int64_t n, int64_t coord_stride,
                        const float* edges, int32_t n_edges, uint8_t* mask_out,
                        void* stream);

/*
 * idx_out[i] = ix + nb*iy with ix = clip(digitize(x_i, edges) - 1, 0, nb-1),
 * likewise iy, nb = n_edges - 1 (digitize with right=False; edges ascending).
 * Bit-exact with square_spaxel_assignment, rubix/telescope/utils.py:78-152
 * (step spaxel_assignment, rubix/core/telescope.py:81-126).
 */
RUBIX_API int rubix_spaxel_assign(const float* coords, int64_t n, int64_t coord_stride,
                        const float* edges, int32_t n_edges, int32_t* idx_out,
                        void* stream);

RUBIX_API size_t rubix_spaxel_sort_workspace_size(int64_t n, int32_t n_segments);

/*
 * Stable sort of particles by spaxel index (LSD radix sort).  Particle i takes
 * part if keep == NULL or keep[i] != 0, and 0 <= idx[i] < n_segments (ids
 * outside are dropped, as jax.ops.segment_sum drops them in calculate_cube,
 * rubix/spectra/ifu.py:286).  perm_out[j] is the original index of the j-th
 * particle in (spaxel, original index) order; the first seg_offsets[n_segments]
 * entries are the kept particles and seg_offsets[s] .. seg_offsets[s+1]-1 are
 * those of spaxel s.  seg_offsets_out has n_segments + 1 entries.
 * Replaces the grouping inside segment_sum (rubix/spectra/ifu.py:286).
 */
RUBIX_API int rubix_spaxel_sort(const int32_t* idx, const uint8_t* keep, int64_t n,
                      int32_t n_segments, int32_t* perm_out, int32_t* seg_offsets_out,
                      void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------- */
/* (b) Fused SSP lookup + mass scaling + Doppler shift/resampling + cube     */
/* ------------------------------------------------------------------------- */

/*
 * Shared inputs of the accumulate kernels.
 *   ssp_flux      [n_met][n_age][n_wave]   SSPGrid.flux (rubix/spectra/ssp/grid.py:28-31)
 *   ssp_metallicity [n_met], ssp_age [n_age]  ascending grids (interp2d x, y)
 *   ssp_wave_z    [n_wave] ascending, the float32 (1+z)*wavelength of
 *                 cosmological_doppler_shift (rubix/spectra/ifu.py:66-80, core/ifu.py:261)
 *   wave_t        [n_wave_t] ascending telescope grid (telescope.wave_seq)
 *   mass, metallicity, age [n]; velocity [n][vel_stride], line-of-sight
 *                 component `vel_component` (rubix_config.yml ifu.doppler)
 *   perm, seg_offsets   output of rubix_spaxel_sort for n_segments spaxels
 */
RUBIX_API size_t rubix_cube_workspace_size(int64_t n, int32_t n_segments, int32_t n_wave_t,
                                           int32_t n_met, int32_t n_age, int32_t n_wave);

/*
 * cube[s][0..n_wave_t) = sum over kept particles p of spaxel s of
 *   resample(mass_p * interp2d_linear(Z_p, age_p), wave_z*exp(v_p/c), wave_t).
 * Replaces calculate_spectra (rubix/core/ifu.py:29-123, ssp.method="linear"),
 * scale_spectrum_by_mass (core/ifu.py:127-159), doppler_shift_and_resampling
 * (core/ifu.py:226-295, spectra/ifu.py:168-266) and calculate_datacube
 * (core/ifu.py:299-341, spectra/ifu.py:270-288), fused; no N x lambda array is
 * materialised.  Deterministic: the same inputs give bit-identical cubes.
 * With n_lsf_taps > 0 (lsf_taps a HOST array of <= 63 taps) every finished
 * spectrum is also convolved along wavelength exactly as rubix_lsf_fwd does with
 * (lsf_taps, n_lsf_taps, lsf_crop); LSF and PSF act on different axes and commute,
 * so a pipeline may fuse its LSF step here and run the PSF afterwards.
 * Limits: n_wave_t <= 4096; n_wave up to about 2600 (shared-memory rows).
 * The workspace (256-byte aligned) must not be shared by calls in flight at the
 * same time.
 */
RUBIX_API int rubix_cube_fwd(const float* ssp_flux, const float* ssp_metallicity,
                   const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                   int32_t n_age, int32_t n_wave, const float* wave_t, int32_t n_wave_t,
                   const float* mass, const float* metallicity, const float* age,
                   const float* velocity, int64_t vel_stride, int32_t vel_component,
                   const int32_t* perm, const int32_t* seg_offsets, int32_t n_segments,
                   int64_t n, const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop,
                   float* cube, int64_t spaxel_stride, void* workspace,
                   size_t workspace_bytes, void* stream);

/*
 * Reads the device error word of the last rubix_cube_fwd that used `workspace`
 * (synchronises `stream`).  *device_error = 1 and RUBIX_E_DEVICE if a shared-memory
 * copy wait in the kernel timed out (the cube is then invalid), else 0 / RUBIX_OK.
 */
RUBIX_API int rubix_cube_status(const void* workspace, int* device_error, void* stream);

/*
 * Replaces, in the dusty pipeline (rubix/config/pipeline_config.yml:97-111), the
 * extinction factor that calculate_extinction (rubix/core/dust.py:53-63 ->
 * rubix/spectra/dust/dust_extinction.py:345-358) multiplies into every resampled
 * spectrum before calculate_datacube sums them.
 *
 * rubix_cube_fwd with every particle's resampled spectrum multiplied by its dust
 * transmission 2^(ext_exponent[t] * av[i]) = 10^(-0.4 A(lambda_t)/A(V) * A_V,i) before
 * the per-spaxel sum.  av[i]: A_V of particle i (input order, rubix_dust_av);
 * ext_exponent[t] = -0.4 * log2(10) * A(lambda_t)/A(V) of the extinction model at the
 * telescope wavelengths (n_wave_t floats).  Same workspace (rubix_cube_workspace_size),
 * limits, determinism and status word as rubix_cube_fwd.
 */
RUBIX_API int rubix_cube_fwd_dust(const float* ssp_flux, const float* ssp_metallicity,
                                  const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                                  int32_t n_age, int32_t n_wave, const float* wave_t,
                                  int32_t n_wave_t, const float* mass, const float* metallicity,
                                  const float* age, const float* velocity, int64_t vel_stride,
                                  int32_t vel_component, const float* av,
                                  const float* ext_exponent, const int32_t* perm,
                                  const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                  const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop,
                                  float* cube, int64_t spaxel_stride, void* workspace,
                                  size_t workspace_bytes, void* stream);

/*
 * The adjoint of rubix_cube_fwd_dust for the particle inputs (what jax.grad through
 * calculate_extinction gives for mass, metallicity, age and velocity; A_V, a function
 * of the coordinates and the gas, is held fixed): rubix_cube_bwd with the cube
 * adjoint seen through each particle's transmission 2^(ext_exponent[t] * av[i]).
 * Same workspace (rubix_cube_bwd_workspace_size) and limits as rubix_cube_bwd.
 */
RUBIX_API int rubix_cube_bwd_dust(const float* ssp_flux, const float* ssp_metallicity,
                                  const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                                  int32_t n_age, int32_t n_wave, const float* wave_t,
                                  int32_t n_wave_t, const float* mass, const float* metallicity,
                                  const float* age, const float* velocity, int64_t vel_stride,
                                  int32_t vel_component, const float* av,
                                  const float* ext_exponent, const int32_t* perm,
                                  const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                  const float* adj, int64_t adj_stride, float* grad_mass,
                                  float* grad_metallicity, float* grad_age, float* grad_vlos,
                                  void* workspace, size_t workspace_bytes, void* stream);

/*
 * rubix_cube_bwd_dust plus grad_av[i] = dL/dA_V of every particle (the derivative of its
 * transmission 2^(ext_exponent[t] * av[i]) in its spectrum), which jax.grad through
 * calculate_extinction (rubix/core/dust.py:53-63) passes on to the column density.
 * Same workspace and limits as rubix_cube_bwd.
 */
RUBIX_API int rubix_cube_bwd_dust_av(const float* ssp_flux, const float* ssp_metallicity,
                                     const float* ssp_age, const float* ssp_wave_z,
                                     int32_t n_met, int32_t n_age, int32_t n_wave,
                                     const float* wave_t, int32_t n_wave_t, const float* mass,
                                     const float* metallicity, const float* age,
                                     const float* velocity, int64_t vel_stride,
                                     int32_t vel_component, const float* av,
                                     const float* ext_exponent, const int32_t* perm,
                                     const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                     const float* adj, int64_t adj_stride, float* grad_mass,
                                     float* grad_metallicity, float* grad_age, float* grad_vlos,
                                     float* grad_av, void* workspace, size_t workspace_bytes,
                                     void* stream);

/*
 * Replaces the per-cell extinction of rubix/spectra/dust/dust_extinction.py:291-306
 * (12 + log10(O/(16 H)), calculate_dust_to_gas_ratio :13-90, calculate_extinction
 * :93-160, divided by the spaxel area).
 *
 * ext_out[i] = mass[i] * DGR(g_i) * scale / spaxel_area with
 * g_i = 12 + log10(metals[i*metals_stride + o_col] / (16 * metals[i*metals_stride + h_col]))
 * and DGR(g) = 1 / 10^(a + alpha * (x_sol - g)); dgr_params = {x_sol, a_hi, alpha_hi,
 * a_lo, alpha_lo, x_transition}: with broken != 0 the (a_lo, alpha_lo) branch applies
 * where g <= x_transition (Remy-Ruyer et al. 2014 broken power law), else (a_hi,
 * alpha_hi) everywhere.  scale = 3 pi (Msun/kpc^2 in g/cm^2) / (0.4 ln10 lambda_V rho_D).
 */
RUBIX_API int rubix_dust_gas_extinction(const float* mass, const float* metals,
                                        int64_t metals_stride, int32_t h_col, int32_t o_col,
                                        int64_t n, const float* dgr_params, int32_t broken,
                                        float scale, float spaxel_area, float* ext_out,
                                        void* stream);

/*
 * Replaces the column-density part of apply_spaxel_extinction
 * (rubix/spectra/dust/dust_extinction.py:262-343): the A_V of every star.
 *
 * Gas cell j: z = gas_coords[j*gas_stride + 2], pixel assignment gas_pa[j], extinction
 * gas_ext[j] (rubix_dust_gas_extinction); star i likewise (star_coords, star_pa).
 * Spaxel of a cell or star: min(pa, n_segments - 1); pa_limit bounds every assignment
 * (pa < pa_limit; (n_edges-1)^2 of the spaxel assignment).  av_out[i] is rubix's value:
 * jnp.interp of the star's z, extrapolating on the left, over its spaxel's cells
 * (z, cumulative extinction in (assignment, z) order) merged with every other cell at
 * (fl32(z * 1e30), 0) in rubix's stable-sort order.  No gas (n_gas = 0) gives 0.
 * Deterministic; about 40 launches; no allocation.
 */
/*
 * Replaces rubix/spectra/dust/dust_extinction.py:345-358 on materialised spectra
 * (rubixdata.stars.spectra * extinction): rows[i*row_stride + t] *=
 * 2^(ext_exponent[t] * av[i]) for i < n, t < n_wave_t.
 */
RUBIX_API int rubix_dust_apply_rows(float* rows, int64_t n, int32_t n_wave_t,
                                    int64_t row_stride, const float* av,
                                    const float* ext_exponent, void* stream);

RUBIX_API size_t rubix_dust_av_workspace_size(int64_t n_gas, int32_t n_segments);
RUBIX_API int rubix_dust_av(const float* gas_coords, int64_t gas_stride, const int32_t* gas_pa,
                            const float* gas_ext, int64_t n_gas, const float* star_coords,
                            int64_t star_stride, const int32_t* star_pa, int64_t n_stars,
                            int32_t n_segments, int32_t pa_limit, float* av_out,
                            void* workspace, size_t workspace_bytes, void* stream);

/*
 * What jax.grad through rubix's column interpolation gives
 * (rubix/spectra/dust/dust_extinction.py:262-343, the jnp.interp of each star's z on
 * the masked cumulative extinction of its spaxel) and through the per-cell extinction
 * (dust_extinction.py:291-306, dust-to-gas ratio of 12 + log10(O/(16 H))).
 *
 * rubix_dust_av_bwd: given grad_av[i] = dL/dA_V of every star, writes
 * grad_star_z[i] = dL/dz of the star (the slope of its interpolation; 0 when clamped)
 * and grad_gas_ext[j] = dL/d ext of every gas cell (the cumulative sums' adjoint); the
 * gas heights are held fixed.  Same inputs and limits as rubix_dust_av; workspace
 * rubix_dust_av_bwd_workspace_size (256-byte aligned).  Deterministic: records are
 * sorted by node and summed in star order (float64).
 */
RUBIX_API size_t rubix_dust_av_bwd_workspace_size(int64_t n_gas, int32_t n_segments,
                                                  int64_t n_stars);
RUBIX_API int rubix_dust_av_bwd(const float* gas_coords, int64_t gas_stride,
                                const int32_t* gas_pa, const float* gas_ext, int64_t n_gas,
                                const float* star_coords, int64_t star_stride,
                                const int32_t* star_pa, int64_t n_stars, int32_t n_segments,
                                int32_t pa_limit, const float* grad_av, float* grad_star_z,
                                float* grad_gas_ext, void* workspace, size_t workspace_bytes,
                                void* stream);

/*
 * The adjoint of rubix_dust_gas_extinction: from grad_ext[j] = dL/d ext of each cell,
 * grad_mass[j] = dL/d mass, grad_h[j] = dL/d metals[j][h_col] and grad_o[j] = dL/d
 * metals[j][o_col] (the other metal columns do not enter).  Same parameters as the
 * forward.
 */
RUBIX_API int rubix_dust_gas_extinction_bwd(const float* mass, const float* metals,
                                            int64_t metals_stride, int32_t h_col,
                                            int32_t o_col, int64_t n, const float* dgr_params,
                                            int32_t broken, float scale, float spaxel_area,
                                            const float* grad_ext, float* grad_mass,
                                            float* grad_h, float* grad_o, void* stream);

/*
 * Replaces the array preparation of rubix/core/fits.py:88-100 (astropy writing
 * datacube.T as a float32 image HDU): out[(l*B + b)*A + a] = the big-endian bit
 * pattern of cube[(a*B + b)*spaxel_stride + l] for a < A, b < B (B <= 65535), l < L,
 * i.e. the bytes of the FITS data array of the cube [A][B][L].
 */
RUBIX_API int rubix_fits_cube_layout(const float* cube, int32_t A, int32_t B, int32_t L,
                                     int64_t spaxel_stride, void* out, void* stream);

/*
 * rubix_psf_fwd and rubix_lsf_fwd with the taps in device memory (ty, tx, taps are
 * device pointers of m_y, m_x, n_taps floats), so that taps computed on the device
 * (rubix_gauss_taps) need no copy to the host.  Same arguments, limits and results
 * (including the TMA staging of 16-byte spaxel rows and rubix_psf_status).
 */
RUBIX_API int rubix_psf_fwd_dtaps(const float* in, float* out, int32_t ny, int32_t nx,
                                  int32_t n_wave_t, int64_t spaxel_stride_in,
                                  int64_t spaxel_stride_out, const float* ty, int32_t m_y,
                                  const float* tx, int32_t m_x, void* stream);
RUBIX_API int rubix_lsf_fwd_dtaps(const float* in, float* out, int64_t n_rows,
                                  int32_t n_wave_t, int64_t row_stride_in,
                                  int64_t row_stride_out, const float* taps, int32_t n_taps,
                                  int32_t crop, void* stream);

/*
 * Replaces, for a sigma held on the device, the tap computation of rubix's
 * gaussian_kernel_2d (telescope/psf/kernels.py:5-31; the 2-D kernel is the outer product
 * of these 1-D taps) and of the LSF kernel (telescope/lsf/lsf.py:12-26), plus the
 * derivative jax.grad takes through them.
 *
 * sigma: one double in device memory; x: m positions (host, copied by value, m < 64).
 * taps[i] = e_i / sum e with e_i = exp(-x_i^2 / (2 sigma^2)); dtaps (optional) = d taps /
 * d sigma; rtaps (optional) = taps reversed, followed by one zero when rtaps_pad (the
 * adjoint taps of a 'same' convolution with even m).  float64 arithmetic, float32
 * results, all in device memory; one launch, no synchronisation.
 */
RUBIX_API int rubix_gauss_taps(const double* sigma, const double* x, int32_t m, float* taps,
                               float* dtaps, float* rtaps, int32_t rtaps_pad, void* stream);


/*
 * No counterpart in rubix (rubix has no C interface; JAX allocates its buffers).
 *
 * rubix_cube_fwd without the workspace argument, for callers that cannot allocate
 * device memory when they render: hosts that own all GPU memory through their own
 * pool and forbid cudaMalloc from plugins, or loops that must never enter an
 * allocator.  Same inputs, output and results as rubix_cube_fwd (bit-identical); the
 * scratch is a static device array of RUBIX_CUBE_NOALLOC_SCRATCH_BYTES that every GPU
 * loading this part of the library keeps until process exit.  Arguments are checked
 * as rubix_cube_fwd checks them (same codes); then problems needing more scratch
 * (rubix_cube_workspace_size) return RUBIX_E_WORKSPACE.  The first call in a CUDA
 * context looks up the array's address (cudaGetSymbolAddress, cached per context)
 * and should come before any stream capture.  All calls share the array: calls whose
 * GPU work overlaps race.
 */
#define RUBIX_CUBE_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
RUBIX_API int rubix_cube_fwd_noalloc(const float* ssp_flux, const float* ssp_metallicity,
                                     const float* ssp_age, const float* ssp_wave_z,
                                     int32_t n_met, int32_t n_age, int32_t n_wave,
                                     const float* wave_t, int32_t n_wave_t, const float* mass,
                                     const float* metallicity, const float* age,
                                     const float* velocity, int64_t vel_stride,
                                     int32_t vel_component, const int32_t* perm,
                                     const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                     const float* lsf_taps, int32_t n_lsf_taps,
                                     int32_t lsf_crop, float* cube, int64_t spaxel_stride,
                                     void* stream);

/*
 * No counterpart in rubix (rubix has no device error word).
 *
 * rubix_cube_status for rubix_cube_fwd_noalloc, whose caller never holds the scratch
 * address: reads the device error word of the last no-alloc call in the current
 * context (synchronises `stream`).  *device_error = 1 and RUBIX_E_DEVICE if a
 * shared-memory copy wait in the kernel gave up (that cube is invalid), else 0 /
 * RUBIX_OK.
 */
RUBIX_API int rubix_cube_noalloc_status(int* device_error, void* stream);

/* ------------------------------------------------------------------------- */
/* Materialised intermediates (step-by-step use; the fused path never needs them) */
/* ------------------------------------------------------------------------- */

/*
 * out[i][k] = interp2d_linear(metallicity_i, age_i) of ssp_flux[:, :, k], times
 * mass_i when mass != NULL; 0 outside the grid.  Replaces the lookup of
 * calculate_spectra (rubix/core/ifu.py:63-121; spectra/ssp/grid.py:113-120 with
 * method="linear") and, with mass, scale_spectrum_by_mass (core/ifu.py:149-157).
 */
RUBIX_API int rubix_ssp_lookup(const float* ssp_flux, const float* ssp_metallicity,
                               const float* ssp_age, int32_t n_met, int32_t n_age,
                               int32_t n_wave, const float* metallicity, const float* age,
                               const float* mass, int64_t n, float* out, int64_t out_stride,
                               void* stream);

/*
 * values[i][0..width) = 0 for every i with mask[i] == 0, in place (rows of `stride`
 * floats): the zeroing of particle fields outside the aperture done by
 * filter_particles, rubix/core/telescope.py:159-172.
 */
RUBIX_API int rubix_mask_zero(float* values, int64_t n, int32_t width, int64_t stride,
                              const uint8_t* mask, void* stream);

/* out[i][k] = rows[i][k] * mass[i]: scale_spectrum_by_mass, rubix/core/ifu.py:149-157. */
RUBIX_API int rubix_scale_rows(const float* rows, int64_t row_stride, const float* mass,
                               int64_t n, int32_t n_wave, float* out, int64_t out_stride,
                               void* stream);

/*
 * resample_spectrum (rubix/spectra/ifu.py:224-266) of each given spectrum row i on the
 * Doppler-shifted grid fl32(ssp_wave_z * fl32(exp(v_i/c))) onto wave_t: the
 * doppler_shift_and_resampling step (rubix/core/ifu.py:226-295) for spectra the caller
 * holds.  n_wave <= ~25000.
 */
RUBIX_API int rubix_resample_rows(const float* spectra, int64_t spectra_stride,
                                  const float* ssp_wave_z, int32_t n_wave,
                                  const float* velocity, int64_t vel_stride,
                                  int32_t vel_component, int64_t n, const float* wave_t,
                                  int32_t n_wave_t, float* out, int64_t out_stride,
                                  void* stream);

/*
 * out[s] = sum of rows[perm[j]] for j in [seg_offsets[s], seg_offsets[s+1]) in that
 * order: calculate_cube (rubix/spectra/ifu.py:270-288) for spectra the caller holds,
 * with (perm, seg_offsets) from rubix_spaxel_sort.
 */
RUBIX_API int rubix_segment_sum_rows(const float* rows, int64_t row_stride, int32_t n_wave_t,
                                     const int32_t* perm, const int32_t* seg_offsets,
                                     int32_t n_segments, float* out, int64_t out_stride,
                                     void* stream);

/* ------------------------------------------------------------------------- */
/* (c) PSF: per-wavelength 2-D convolution, separable Gaussian               */
/* ------------------------------------------------------------------------- */

/*
 * out[y][x][l] = sum_{i,j} ty[i] tx[j] in[y + oy - i][x + ox - j][l] with zero
 * padding, oy = (m_y-1)/2, ox = (m_x-1)/2 ("same" mode of convolve2d).  ty/tx are
 * HOST arrays of m_y/m_x taps (m_y <= 31, m_x <= 63).  With ty = tx = the normalised 1-D
 * Gaussian this equals convolve2d(plane, gaussian_kernel_2d, mode="same") for every
 * plane: apply_psf, rubix/telescope/psf/psf.py:33-58 with kernels.py:5-31 (step
 * convolve_psf, rubix/core/psf.py:15-75).  in and out must not overlap.
 */
RUBIX_API int rubix_psf_fwd(const float* in, float* out, int32_t ny, int32_t nx, int32_t n_wave_t,
                  int64_t spaxel_stride_in, int64_t spaxel_stride_out, const float* ty,
                  int32_t m_y, const float* tx, int32_t m_x, void* stream);
/*
 * With m_y = m_x <= 17, a 16-byte aligned `in` and spaxel_stride_in a multiple of 4
 * floats (e.g. n_wave_t rounded up to a multiple of 4), the input rows are staged by
 * tiled TMA copies; a staged-row wait that runs out (about 1 s) makes the kernel set a
 * device error word and return.  rubix_psf_status reads that word (synchronises
 * `stream`): *device_error = 1 and RUBIX_E_DEVICE if it was set since the last read,
 * which clears it; 0 and RUBIX_OK otherwise.
 */
RUBIX_API int rubix_psf_status(int* device_error, void* stream);

/* ------------------------------------------------------------------------- */
/* (d) LSF: 1-D convolution along wavelength                                 */
/* ------------------------------------------------------------------------- */

/*
 * out[r][t] = sum_j taps[j] * in[r][t + crop - j] (zero outside [0, n_wave_t)):
 * the full convolution cropped to [crop, n_wave_t + crop).  taps is a HOST array
 * of n_taps <= 255 values.  With the rubix Gaussian taps and crop = 12 this is
 * apply_lsf, rubix/telescope/lsf/lsf.py:29-105 (step convolve_lsf,
 * rubix/core/lsf.py:14-67).  in and out must not overlap.
 */
RUBIX_API int rubix_lsf_fwd(const float* in, float* out, int64_t n_rows, int32_t n_wave_t,
                  int64_t row_stride_in, int64_t row_stride_out, const float* taps,
                  int32_t n_taps, int32_t crop, void* stream);

/* ------------------------------------------------------------------------- */
/* Adjoints (gradients of a loss L of the cube)                              */
/* ------------------------------------------------------------------------- */

/*
 * The gradient of the datacube with respect to the particle inputs that rubix
 * obtains with jax.grad through calculate_spectra -> scale_spectrum_by_mass ->
 * doppler_shift_and_resampling -> calculate_datacube (rubix/core/ifu.py:29-341;
 * RubixPipeline.gradient, rubix/core/pipeline.py:204-208).
 * adj[s][t] (row stride adj_stride) = dL/dcube[s][t] of the cube rubix_cube_fwd
 * writes WITHOUT its LSF epilogue (apply the PSF and LSF adjoints to dL/dcube first:
 * rubix_psf_fwd / rubix_lsf_fwd with reversed taps).  Writes, for every particle
 * i < n (zero for particles outside the sorted set), dL/dmass_i, dL/dmetallicity_i,
 * dL/dage_i and dL/dv_i of the line-of-sight velocity component; any of the four
 * output pointers may be NULL.  Derivatives hold the float32 bracket choices and the
 * in-range wavelength mask fixed, as automatic differentiation of the forward
 * formulas does; particles with T' = 0 or a non-finite T/T' get zero gradients.
 * Same inputs and limits as rubix_cube_fwd; deterministic.
 */
RUBIX_API size_t rubix_cube_bwd_workspace_size(int64_t n, int32_t n_segments, int32_t n_wave_t,
                                               int32_t n_met, int32_t n_age, int32_t n_wave);
RUBIX_API int rubix_cube_bwd(const float* ssp_flux, const float* ssp_metallicity,
                             const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                             int32_t n_age, int32_t n_wave, const float* wave_t,
                             int32_t n_wave_t, const float* mass, const float* metallicity,
                             const float* age, const float* velocity, int64_t vel_stride,
                             int32_t vel_component, const int32_t* perm,
                             const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                             const float* adj, int64_t adj_stride, float* grad_mass,
                             float* grad_metallicity, float* grad_age, float* grad_vlos,
                             void* workspace, size_t workspace_bytes, void* stream);

/*
 * No counterpart in rubix (jax.grad reduces inside XLA).
 * *out (device double) = sum_i a[i] * b[i]: per-thread float partial sums, double
 * block and grid reductions in a fixed order (deterministic).  Used for the
 * gradients with respect to the PSF and LSF widths, <dL/dcube, d cube/d sigma>.
 * The workspace (rubix_dot_workspace_size bytes, 8-byte aligned) must not be shared
 * by calls in flight at the same time.
 */
RUBIX_API size_t rubix_dot_workspace_size(void);
RUBIX_API int rubix_dot(const float* a, const float* b, int64_t n, double* out, void* workspace,
                        size_t workspace_bytes, void* stream);

/*
 * No counterpart in rubix (jax.grad forms these inner products inside XLA).
 * Fused forms of rubix_dot(w, conv(in)) for the σ gradients, the convolution never
 * written to memory: *out (device double) = sum over the cube of w * PSF(in) with the
 * device taps ty (y) and tx (x) of rubix_psf_fwd_dtaps (m odd, <= 21), or
 * sum over rows of w * LSF(in) with the device taps of rubix_lsf_fwd_dtaps
 * (n_taps <= 28).  The convolution is computed with the same arithmetic as those
 * entry points; per-thread float partial sums, double block sums added in block order
 * (deterministic).  The workspace (rubix_fused_dot_workspace_size bytes, 8-byte
 * aligned) must not be shared by calls in flight at the same time.  Other tap counts
 * return RUBIX_E_UNSUPPORTED.
 */
RUBIX_API size_t rubix_fused_dot_workspace_size(void);
RUBIX_API int rubix_psf_dot_dtaps(const float* in, int64_t spaxel_stride_in, const float* w,
                                  int64_t spaxel_stride_w, int32_t ny, int32_t nx,
                                  int32_t n_wave_t, const float* ty, const float* tx, int32_t m,
                                  double* out, void* workspace, size_t workspace_bytes,
                                  void* stream);
RUBIX_API int rubix_lsf_dot_dtaps(const float* in, int64_t n_rows, int32_t n_wave_t,
                                  int64_t row_stride_in, const float* w, int64_t row_stride_w,
                                  const float* taps, int32_t n_taps, int32_t crop, double* out,
                                  void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------- */
/* Ragged batches of galaxies                                                */
/* ------------------------------------------------------------------------- */
/*
 * No counterpart in rubix (rubix renders one galaxy per pipeline run,
 * rubix/core/pipeline.py:137-170).  A batch of n_gal galaxies shares the SSP grid and
 * the telescope wavelength grid; galaxy g owns particles [particle_offsets[g],
 * particle_offsets[g+1]) and the square S_g x S_g spaxel grid stored as global spaxels
 * [seg_base[g], seg_base[g] + S_g^2) of one concatenated cube.  All table arguments
 * are DEVICE arrays.  With global spaxel ids the ordinary rubix_spaxel_sort,
 * rubix_cube_fwd / rubix_cube_bwd (n_segments = seg_base[n_gal]) and rubix_lsf_fwd
 * process the whole batch in one launch each.
 */

/*
 * Per particle: spaxel assignment with its galaxy's ascending bin edges
 * (edges[edge_offsets[g] .. edge_offsets[g+1])), as rubix_spaxel_assign; keep_out = 1
 * when inside the galaxy's aperture [edges[0], edges[-1]] (as rubix_aperture_mask)
 * and when the flat id is below S_g^2; idx_out = seg_base[g] + flat id (0 when not
 * kept).
 */
RUBIX_API int rubix_ragged_assign(const float* coords, int64_t n, int64_t coord_stride,
                                  const int64_t* particle_offsets, int32_t n_gal,
                                  const float* edges, const int32_t* edge_offsets,
                                  const int32_t* sbin, const int64_t* seg_base, int32_t* idx_out,
                                  uint8_t* keep_out, void* stream);

/*
 * rubix_psf_fwd for every galaxy of a batch in one launch.  taps [n_gal][2][m]: the
 * y and x taps of each galaxy zero-padded and centred to the odd size m <= 21.
 * block_offsets[g] = sum over g' < g of ceil(S_g'/32) * ceil(n_wave_t/32) and
 * n_blocks = block_offsets[n_gal] (host copy).
 */
RUBIX_API int rubix_ragged_psf_fwd(const float* in, float* out, int32_t n_wave_t,
                                   int64_t spaxel_stride_in, int64_t spaxel_stride_out,
                                   int32_t n_gal, const int32_t* sbin, const int64_t* seg_base,
                                   const int32_t* block_offsets, int32_t n_blocks,
                                   const float* taps, int32_t m, void* stream);

/*
 * out[g] (device doubles) = sum over i in [offsets[g], offsets[g+1]) of a[i] * b[i];
 * deterministic (fixed split and order).  n_seg <= 65535.
 */
RUBIX_API size_t rubix_segmented_dot_workspace_size(int32_t n_seg);
RUBIX_API int rubix_segmented_dot(const float* a, const float* b, const int64_t* offsets,
                                  int32_t n_seg, double* out, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------- */
/* Galaxy orientation                                                        */
/* ------------------------------------------------------------------------- */
/*
 * rotate_galaxy (rubix/core/rotation.py:11-117, galaxy/alignment.py:66-265):
 *   rubix_inertia_tensor: out9 (device, float64, row-major 3x3) = the moment-of-inertia
 *     tensor of the particles with |x| <= halfmass_radius (moment_of_inertia_tensor,
 *     alignment.py:66-120), including the index padding of rubix's
 *     jnp.where(..., size=N): particle 0 counts once more for every particle outside.
 *   rubix_rotate_vectors: out[i] = in[i] . M (row vectors times the host row-major 3x3
 *     float64 matrix, float64 arithmetic rounded once; in and out may alias).
 * The caller diagonalises the tensor (eigh, eigenvectors in ascending eigenvalue order)
 * and composes M = R_inertia . R_euler on the host.
 */
RUBIX_API size_t rubix_inertia_workspace_size(void);
RUBIX_API int rubix_inertia_tensor(const float* positions, int64_t n, int64_t stride,
                                   const float* masses, float halfmass_radius, double* out9,
                                   void* workspace, size_t workspace_bytes, void* stream);
RUBIX_API int rubix_rotate_vectors(const float* in, float* out, int64_t n, int64_t stride_in,
                                   int64_t stride_out, const double* matrix9, void* stream);

/*
 * rotate_galaxy + filter_particles + spaxel_assignment of one particle component in one
 * pass (replaces the rotate_vectors / aperture-mask / masked-copy / assignment launches
 * of rubix/core/rotation.py:66-113, rubix/core/telescope.py:151-199 and
 * rubix/core/telescope.py:81-126 when the three steps run back to back):
 *   coords, velocity: [n][3] float32, contiguous;
 *   matrix9: host row-major 3x3 float64 M, or NULL for no rotation; with M,
 *     coords_out[i] = coords[i] . M and velocity_out[i] = velocity[i] . M (as
 *     rubix_rotate_vectors; out may alias in), and the turned coordinates are the ones
 *     masked and assigned;
 *   mask_out[i] = 1 inside the inclusive aperture [min(edges), max(edges)]^2 (as
 *     rubix_aperture_mask); may be NULL when n_fields == 0;
 *   fields: n_fields (<= 8) float32 per-particle arrays of field_widths[f] values each
 *     (host arrays of device pointers), copied to fields_out[f] with the particles
 *     outside set to 0 (filter_particles; out may alias in);
 *   idx_out[i] = the flat spaxel index of the (turned) coordinates (as
 *     rubix_spaxel_assign).
 */
RUBIX_API int rubix_orient_filter_assign(const float* coords, const float* velocity, int64_t n,
                                         const double* matrix9, float* coords_out,
                                         float* velocity_out, const float* edges,
                                         int32_t n_edges, int32_t n_fields,
                                         const float* const* fields_in,
                                         float* const* fields_out,
                                         const int32_t* field_widths, uint8_t* mask_out,
                                         int32_t* idx_out, void* stream);

/* ------------------------------------------------------------------------- */
/* Observation noise                                                         */
/* ------------------------------------------------------------------------- */
/*
 * apply_noise (rubix/core/noise.py:17-80; calculate_S2N / calculate_noise_cube,
 * rubix/telescope/noise/noise.py:35-115) in three calls:
 *   rubix_flux_image:   flux[s] = sum_t cube[s][t]
 *   rubix_noise_median: *median (device) = median of flux, or 0 when any flux <= 0
 *                       (rubix's jnp.median over where(flux > 0, flux, nan) is NaN then,
 *                       and nan_to_num makes it 0)
 *   rubix_apply_noise:  cube[s][t] += cube[s][t] * z * sqrt(median) / s2n / sqrt(flux[s])
 *                       (0 where flux <= 0), z ~ N(0,1) (distribution 0) or U[0,1) (1).
 * rubix draws z from jax.random with a fixed key; here z comes from Philox4x32-10 keyed
 * by `seed` with the element index as counter: reproducible per seed, equal to rubix's
 * noise in distribution only.
 */
RUBIX_API int rubix_flux_image(const float* cube, int64_t n_spaxels, int32_t n_wave_t,
                               int64_t spaxel_stride, float* flux, void* stream);
RUBIX_API size_t rubix_noise_median_workspace_size(void);
RUBIX_API int rubix_noise_median(const float* flux, int64_t n, float* median, void* workspace,
                                 size_t workspace_bytes, void* stream);
RUBIX_API int rubix_apply_noise(float* cube, int64_t n_spaxels, int32_t n_wave_t,
                                int64_t spaxel_stride, const float* flux, const float* median,
                                float signal_to_noise, int32_t distribution, uint64_t seed,
                                void* stream);
/* No counterpart in rubix: the generator of rubix_apply_noise on the host (one block of
 * Philox4x32-10: counter[4], key[2] -> out[4]), for checking its output. */
RUBIX_API int rubix_philox4x32_10(const uint32_t* counter4, const uint32_t* key2, uint32_t* out4);

/* ------------------------------------------------------------------------- */
/* Tuning                                                                    */
/* ------------------------------------------------------------------------- */
/*
 * No counterpart in rubix.  Work-item shape of rubix_cube_fwd / rubix_cube_bwd on a
 * device: spaxels are processed in chunks of `chunk` particles (multiple of 32 in
 * [32, 256]; default 256) and single-chunk spaxels with at least `big_item` particles
 * are scheduled first (default 64).  Results do not depend on big_item; they depend
 * on chunk only through the summation order of spaxels longer than one chunk.
 * Workspace sizes follow the tuning current at query time.  A per-device table
 * guarded by a mutex; set_(device, NULL) restores the defaults.
 */
typedef struct {
  int32_t chunk;
  int32_t big_item;
} rubix_cube_tuning;
RUBIX_API int rubix_cube_tuning_set(int32_t device, const rubix_cube_tuning* tuning);
RUBIX_API int rubix_cube_tuning_get(int32_t device, rubix_cube_tuning* tuning);

#ifdef __cplusplus
}
#endif

#endif /* RUBIX_GB300_H */
