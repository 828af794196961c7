/*
 * mpsq.h — C ABI of libmpsq.so, the GB300 (sm_103a) engine for the S(Q,omega) path of
 * MP_TOOLS mp_sqom (per-frame, per-species type-1 NUFFT of atom positions onto a
 * Brillouin-zone Q grid, species weighting, windowed time transform, |F|^2 sums).
 *
 * Three layers, all plain C types (no CUDA or torch types cross this boundary except an
 * opaque stream handle passed as void*):
 *
 *  1. Link-compatible replacements of the FINUFFT type-1 entry points that mp_sqom and mp_sql
 *     call.  Host pointers in, host pointers out, synchronous.  A Fortran program that links
 *     -lmpsq instead of -lfinufft runs unchanged.
 *  2. A guru-style plan API (makeplan / setpts / execute / destroy) on DEVICE pointers, the
 *     batched operator the loops around the call are rebuilt on.
 *  3. The S(Q,omega) job API: a device-resident trajectory of frames goes in, the loops of
 *     mp_sqom's frame_loop / plot_loop (selection, phases, strengths, NUFFT, species weights,
 *     elastic mean, total S(Q), E=const maps, E(Q) dispersion cuts, Gaussian-window spectra)
 *     run on the GPU, maps come out.
 *
 * Every function returns 0 on success and a nonzero MPSQ_ERR_* code on failure; the text of
 * the last failure of the calling thread is available from mpsq_last_error().  The Fortran
 * entry points report the same code through their `ier` argument.  There is no CPU fallback:
 * without a usable CUDA device every compute call fails with MPSQ_ERR_CUDA.
 */
#ifndef MPSQ_H
#define MPSQ_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
#define MPSQ_OK            0
#define MPSQ_ERR_ARG       1   /* invalid argument (size, pointer, option)              */
#define MPSQ_ERR_ALLOC     2   /* device or pinned-host allocation failed               */
#define MPSQ_ERR_CUDA      3   /* CUDA runtime error (no device, launch failure, ...)   */
#define MPSQ_ERR_CUFFT     4   /* cuFFT plan or execution failure                       */
#define MPSQ_ERR_STATE     5   /* call out of order (e.g. execute before setpts)        */
#define MPSQ_ERR_DEVICE    6   /* a kernel reported an internal bound violation         */

/* ---- precision ---------------------------------------------------------------------- */
#define MPSQ_FP32          0   /* split precision: FP64-exact phase reduction, FP32 spread/FFT */
#define MPSQ_FP64          1   /* plain FP64 throughout                                   */

/* ---- 1. FINUFFT-compatible entry points -------------------------------------------
 *
 * Semantics (FINUFFT type 1, default mode order):
 *   fk[(k1+ms/2) + ms*(k2+mt/2) (+ ms*mt*(k3+mu/2))] =
 *       sum_j cj[j] * exp(i*sgn(iflag)*(k1*xj[j] + k2*yj[j] (+ k3*zj[j])))
 *   for -m/2 <= k <= (m-1)/2 in each dimension; points anywhere in [-3pi, 3pi) (folded
 *   periodically).  Complex arrays are interleaved (re, im) pairs, i.e. C99 double _Complex
 *   or Fortran complex(8).  opts may be NULL (library defaults); a non-NULL opts is accepted
 *   and ignored.  The relative l2 error of fk is at most about eps (eps is clamped to
 *   [1e-14, 1e-1]) for FP64; FP32 transforms clamp eps to [1e-7, 1e-1] (kernel widths 2..8;
 *   at 1e-7 the relative l2 error is a few 1e-7, set by FP32 rounding).
 */

/* Replaces FINUFFT's C entry finufft2d1 — the routine mp_sqom calls once per frame and
 * species at code/src/mp_sqom56.f90:1148 and mp_sql once per z-layer at
 * code/src/mp_sql56.f90:1129 (through the Fortran wrapper below). */
int finufft2d1(int64_t nj, double* xj, double* yj, double* cj, int iflag, double eps,
               int64_t ms, int64_t mt, double* fk, void* opts);

/* Replaces FINUFFT's finufft3d1, the 3D operator that mp_sql builds as a stack of
 * finufft2d1 slices with z-phased strengths (code/src/mp_sql56.f90:1106-1131). */
int finufft3d1(int64_t nj, double* xj, double* yj, double* zj, double* cj, int iflag,
               double eps, int64_t ms, int64_t mt, int64_t mu, double* fk, void* opts);

/* Single-precision counterparts (FINUFFT's finufftf2d1 / finufftf3d1): float positions,
 * interleaved float complex strengths and modes, FP32 spread/FFT with FP64 phase reduction. */
int finufftf2d1(int64_t nj, float* xj, float* yj, float* cj, int iflag, float eps,
                int64_t ms, int64_t mt, float* fk, void* opts);
int finufftf3d1(int64_t nj, float* xj, float* yj, float* zj, float* cj, int iflag,
                float eps, int64_t ms, int64_t mt, int64_t mu, float* fk, void* opts);

/* Fortran (gfortran, implicit interface, all arguments by reference) entry points, the exact
 * symbols an unmodified mp_sqom / mp_sql links against:
 *   call finufft2d1(n_fft,xf,yf,cf,iflag,eps_fft,n_qx8,n_qy8,ampl_tot,nul_opt,ier)
 * at code/src/mp_sqom56.f90:1148 (types declared at :94-98, :195-196) and
 * code/src/mp_sql56.f90:1129.  `opts` is the address of an unallocated allocatable in the
 * reference (NULL); any value is ignored. */
void finufft2d1_(const int64_t* nj, const double* xj, const double* yj, const double* cj,
                 const int* iflag, const double* eps, const int64_t* ms, const int64_t* mt,
                 double* fk, const void* opts, int* ier);
void finufft3d1_(const int64_t* nj, const double* xj, const double* yj, const double* zj,
                 const double* cj, const int* iflag, const double* eps, const int64_t* ms,
                 const int64_t* mt, const int64_t* mu, double* fk, const void* opts, int* ier);

/* ---- 2. plan API on device pointers ------------------------------------------------ */
typedef struct mpsq_nufft_plan mpsq_nufft_plan;

/* dim = 2 or 3; n_modes[dim]; precision MPSQ_FP32/MPSQ_FP64; ntrans transforms share the
 * points (strength vectors stacked).  stream is a cudaStream_t (NULL = default stream).
 * Mirrors FINUFFT's finufft_makeplan(type=1, ...). */
int mpsq_nufft_makeplan(int dim, const int64_t* n_modes, int iflag, int ntrans, double eps,
                        int precision, void* stream, mpsq_nufft_plan** plan);
/* Device arrays of nj coordinates (float for FP32 plans, double for FP64 plans); z ignored
 * for dim 2.  The points are binned here; the arrays may be freed after the call. */
int mpsq_nufft_setpts(mpsq_nufft_plan* plan, int64_t nj, const void* x, const void* y,
                      const void* z);
/* c: device, ntrans*nj interleaved complex; fk: device, ntrans*prod(n_modes) complex in
 * FINUFFT mode order.  Asynchronous on the plan's stream. */
int mpsq_nufft_execute(mpsq_nufft_plan* plan, const void* c, void* fk);
int mpsq_nufft_destroy(mpsq_nufft_plan* plan);
/* Spreading width and fine-grid size chosen for a plan (for reports and tests). */
int mpsq_nufft_info(const mpsq_nufft_plan* plan, int* width, int64_t* fine_grid);
/* Synchronises the plan's stream and reports a bound violation flagged by its kernels. */
int mpsq_nufft_check_error(mpsq_nufft_plan* plan);

/* ---- 3. S(Q,omega) job API ---------------------------------------------------------- */
#define MPSQ_MAX_SPECIES   16

#define MPSQ_CELL          0   /* positions in lattice units, supercell, vacancies at (0,0,0) */
#define MPSQ_BULK          1   /* positions in Angstrom, one box                             */

#define MPSQ_WEIGHT_UNIT   1   /* j_weight = 1 */
#define MPSQ_WEIGHT_NEUTRON 2  /* j_weight = 2: b_coh per species */
#define MPSQ_WEIGHT_XRAY   3   /* j_weight = 3: 4-Gaussian form factor f(|Q|) per species */

#define MPSQ_FF_MP_SQOM    0   /* f = c + sum a_i exp(-b_i |Q|^2/16), as mp_sqom56.f90:925,931 */
#define MPSQ_FF_STANDARD   1   /* f = c + sum a_i exp(-b_i (|Q|/4pi)^2), as mp_sql56.f90:1052,1056 */

typedef struct mpsq_job_desc {
  int32_t ndim;              /* 2 = Q plane (mp_sqom), 3 = Q volume                       */
  int32_t precision;         /* MPSQ_FP32 or MPSQ_FP64                                    */
  double  eps;               /* NUFFT tolerance                                          */
  int64_t n_modes[3];        /* (n_qx, n_qy, n_qz); n_qz ignored for ndim 2               */
  int32_t input_method;      /* MPSQ_CELL or MPSQ_BULK                                    */
  int32_t phase_rounding;    /* 0: phases from FP32 positions in FP64; 1: as mp_sqom,
                                FP32 dot product times FP32 scale (mp_sqom56.f90:1115)     */
  double  axis[3][3];        /* unit vectors e1, e2, e3 (rows); e3 = ev for ndim 2        */
  double  tpe[3];            /* phase per length unit along each axis (tpe1, tpe2, tpev)  */
  double  centre[3];         /* at_pos_centre                                            */
  int32_t use_range;         /* 1: apply the real-space selection below                  */
  double  pos_min[3];        /* at_pos_min (CELL: compared with the cell index, BULK: r)  */
  double  pos_max[3];        /* at_pos_max                                               */
  double  eps_x;             /* BULK tolerance at the box edge (mp_sqom eps_x)           */
  int32_t bulk_nsuper1;      /* BULK with n_row = 1 1 1 (tolerance eps_x, else 1)        */
  int32_t n_row[3];          /* supercell size (CELL selection by cell index)            */
  double  q_center[3];       /* strengths exp(-i 2pi q_center . r)                      */
  int32_t spatial_window;    /* j_wind: multiply strengths by (1+cos x)(1+cos y)[(1+cos z)]
                                and the amplitudes by 1/4 (1/8 in 3D)                     */
  int32_t n_species;         /* n_atom (species)                                         */
  int64_t species_offset[MPSQ_MAX_SPECIES + 1]; /* atom index ranges within a frame      */
  int32_t mask[MPSQ_MAX_SPECIES];   /* at_mask                                            */
  int32_t weight_mode;       /* MPSQ_WEIGHT_*                                            */
  double  b_coh[MPSQ_MAX_SPECIES];  /* scattering length per species (10^-12 cm)          */
  double  xff[MPSQ_MAX_SPECIES][9]; /* a1 b1 a2 b2 a3 b3 a4 b4 c per species              */
  int32_t ff_convention;     /* MPSQ_FF_MP_SQOM or MPSQ_FF_STANDARD                      */
  double  qphys_origin[3];   /* physical Q (1/Angstrom) of mode (0,0,0) ...              */
  double  qphys_step[3][3];  /* ... plus k_a * qphys_step[a] for mode (k1,k2,k3)         */
  double  qphys_extra_sq;    /* |Q_perp|^2 added to |Q|^2 (mp_sqom's q_vp term, :924)    */
  int64_t n_atoms_frame;     /* n_tot: atoms per frame (float4 records x,y,z,charge)     */
  int32_t n_frames;          /* frames in the trajectory                                 */
  int32_t store_species;     /* 1: also keep per-species amplitudes (atom-pair mode)     */
  int32_t no_pack;           /* 0: when all strengths are real (q_center = 0) two species
                                share one complex fine grid (re/im); 1: never pack        */
  int32_t no_pruned_fft;     /* 0: FP32 volumes use the pruned three-pass fine-grid
                                transform fused with the deconvolution; 1: cuFFT + separate
                                deconvolution                                             */
  int32_t stream_ordered;    /* 1: the job's device memory is allocated and freed in the order
                                of its stream (stream-ordered allocation from the device's
                                memory pool), so creating and destroying a job never waits
                                for the device (concurrent jobs of a request server); one
                                frame lane.  0: plain allocation, destroy waits for the job */
  int64_t q_slab;            /* 0: the amplitude store holds every Q mode.  > 0 (3D only): it
                                holds a slab of at most q_slab kz planes (n_qx n_qy q_slab
                                modes per frame), chosen by mpsq_job_set_q_slab; transforms
                                and maps then cover that slab (jobs whose full store would not
                                fit in device memory run slab by slab)                      */
} mpsq_job_desc;

typedef struct mpsq_job mpsq_job;

/* Allocates the device trajectory, fine grids, amplitude store cs(t,Q) and work buffers.
 * stream is a cudaStream_t (NULL = default). */
int mpsq_job_create(const mpsq_job_desc* desc, void* stream, mpsq_job** job);
int mpsq_job_destroy(mpsq_job* job);
/* Bytes of device memory the job would hold (admission control); no allocation. */
int mpsq_job_estimate_bytes(const mpsq_job_desc* desc, int64_t* bytes);

/* Frames [first, first+count) of float4 atom records (x, y, z, charge), frame-major,
 * n_atoms_frame each.  host != 0: pos is host memory (copied H2D, pinned if possible);
 * host == 0: pos is a device pointer (copied D2D). */
int mpsq_job_set_frames(mpsq_job* job, const float* pos, int32_t first, int32_t count,
                        int host);
/* The same copy issued on `stream` (a cudaStream_t other than the job's, so that uploads of
 * later frames overlap the transform of earlier ones).  The caller orders it against the job's
 * stream, e.g. with an event recorded after the copy and waited on before mpsq_job_transform
 * of those frames; host memory should be pinned for the copy to run asynchronously. */
int mpsq_job_set_frames_on(mpsq_job* job, const float* pos, int32_t first, int32_t count,
                           int host, void* stream);
/* Optional cell indices at_ind (int32 x4 per atom, frame independent) for CELL selection. */
int mpsq_job_set_cell_index(mpsq_job* job, const int32_t* at_ind, int host);

/* Runs the NUFFT of frames [first, first+count) for all selected species and stores the
 * species-weighted amplitudes cs(t,Q) (and per-species ones if requested). */
int mpsq_job_transform(mpsq_job* job, int32_t first, int32_t count);

/* Device pointer to cs(t,Q): complex, n_frames x n_Q, Q index x fastest. */
int mpsq_job_amplitudes(mpsq_job* job, void** cs_dev);

/* Total S(Q) = sum_t |cs(t,Q)|^2 / n_frames / norm2  (mp_sqom56.f90:1381-1387,1573-1574).
 * out: n_Q floats; host != 0 copies to host memory. */
int mpsq_job_sq_total(mpsq_job* job, double norm2, float* out, int host);

/* E=const map for frequency bin j_freq (1-based as in mp_sqom): sliding window of n_int
 * frames, window t_wind[n_int], phases exp(-2pi i (j_freq-1)(i-n_int/2-1)/n_int), mean
 * subtracted, optional 1/|Q| scaling (q2_norm != NULL, n_Q floats), normalised by
 * scale (mp_sqom56.f90:1437-1478,1527,1575-1576).  out: n_Q floats. */
int mpsq_job_sqw_econst(mpsq_job* job, int32_t n_int, const float* t_wind, int32_t j_freq,
                        const float* q2_norm, double scale, float* out, int host);

/* E(Q) dispersion cut: for each of n_path Q indices, sum over start frames of
 * |FFT_n_int(window * cs)|^2 for bins 0..n_freq-1 (mp_sqom56.f90:1480-1517).
 * out: n_path x n_freq floats (frequency fastest). */
int mpsq_job_sqw_dispersion(mpsq_job* job, int32_t n_int, const float* t_wind,
                            int32_t n_path, const int64_t* q_index, int32_t n_freq,
                            const float* q2_norm, double scale, float* out, int host);

/* Atom-pair forms of the two maps above (mp_sqom's j_atc1/j_atc2 option,
 * code/src/mp_sqom56.f90:1460-1464 and :1494-1499): the series is the sum of the raw
 * (unweighted, not mean-subtracted) amplitudes of species sp1 and sp2 (0-based), so the job
 * must have been created with store_species = 1. */
int mpsq_job_sqw_econst_pair(mpsq_job* job, int32_t n_int, const float* t_wind, int32_t j_freq,
                             int32_t sp1, int32_t sp2, double scale, float* out, int host);
int mpsq_job_sqw_dispersion_pair(mpsq_job* job, int32_t n_int, const float* t_wind,
                                 int32_t n_path, const int64_t* q_index, int32_t n_freq,
                                 int32_t sp1, int32_t sp2, double scale, float* out, int host);

/* Intermediate scattering function I(Q,t) (mp_sqom's j_sq != 1 branch) on the mean-subtracted,
 * optionally 1/|Q|-scaled amplitudes x:
 *   map at lag `lag` (:1467-1472): out[q] = Re sum_{i<n_int} x(i+lag) conj(x(i)) / n_int * scale
 *   along a path (:1504-1510):     out[p*n_lag + t] = Re sum_{i<n_int} x(t+i) conj(x(i)) * scale,
 *                                  t < n_lag = n_frames - n_int + 1 (:699). */
int mpsq_job_iqt(mpsq_job* job, int32_t n_int, int32_t lag, const float* q2_norm, double scale,
                 float* out, int host);
int mpsq_job_iqt_dispersion(mpsq_job* job, int32_t n_int, int32_t n_path, const int64_t* q_index,
                            const float* q2_norm, double scale, float* out, int host);

/* Gaussian-window spectrum over the whole run: for every Q, |sum_t g_t (cs - <cs>)
 * exp(-2pi i k t/n_frames)|^2 for k = 0..n_freq-1, g_t = exp(-4 ln2 (t-tc)^2/fwhm^2).
 * n_frames must be a power of two <= 1024.  out: n_freq x n_Q floats (Q fastest). */
int mpsq_job_sqw_gauss(mpsq_job* job, double fwhm_frames, int32_t n_freq,
                       const float* q2_norm, double scale, float* out, int host);

/* Spherical |Q| histogram of species pair products, mp_sql's Gauss integration
 * (code/src/mp_sql56.f90:1224-1254): for every frame and every mode k with
 * |Q| <= q_range, bin = nint(|Q| / q_step),
 * out[(a*n_species + b)*n_hist + bin] += Re(A_a(k) conj(A_b(k))) with A_s the per-species
 * amplitudes (job created with store_species = 1, or the weighted amplitude when
 * n_species = 1) times `amp_scale`.  |Q| is formed in FP32 exactly as the reference's
 * q_norm (code/src/mp_sql56.f90:1041): v = k * d_q per axis, Q = a_cell_inv v (row-major
 * 3x3, left-to-right sums), |Q| by the scaled sum of squares of Fortran NORM2, with no
 * fused multiply-adds, so that modes on a bin edge land in the reference's bin.
 * out: n_species^2 x n_hist doubles. */
int mpsq_job_radial_hist(mpsq_job* job, const double* a_cell_inv, const double* d_q,
                         double q_step, double q_range, int32_t n_hist, double amp_scale,
                         double* out, int host);

/* mp_sqom's speckle filter of a finished map (code/src/mp_sqom56.f90:1531-1570), applied by
 * the reference when s_trig > 0 before the map's (sum N)^2 / t_step normalisation.  The map is
 * n_fast x n_slow floats (n_fast contiguous): walking the flattened map with wrap-around
 * neighbours, a value below min(left, right) / s_trig becomes that minimum and a value above
 * s_trig * max(left, right) that maximum, left being the already filtered predecessor and
 * right the unfiltered successor; perpendicular != 0 (E=const, total and I(Q,t) plane maps)
 * repeats the walk over the transposed map, perpendicular = 0 is the E(Q) cut
 * (n_fast = frequencies).  Bit-identical to the sequential walk.  The result is multiplied
 * by post_scale.  host != 0: map is a host array, else a device array (in place, on
 * `stream`).  Synchronous.  Replaces the filter loops of code/src/mp_sqom56.f90:1541-1567. */
int mpsq_speckle_filter(float* map, int64_t n_fast, int64_t n_slow, float s_trig,
                        int32_t perpendicular, float post_scale, int32_t host, void* stream);

/* One-phonon mode (mp_sqom's j_oneph = 1, code/src/mp_sqom56.f90:1037-1098; "for verification"),
 * replacing mpsq_job_transform for frames [first, first+count): per species, the in-plane
 * displacements d = r - at_base - cell (+ n_row/2) summed per cell column into u_x, u_y on the
 * n_row x n_row cell grid, 2D FFT (exp(-i), unscaled) / n_row, and for Q pixel
 * ((ii-1) n_row + k, (jj-1) n_row + l) of the n_bz x n_bz zones
 *   A_j = exp(-2 pi i (q_x b_x + q_y b_y)) (q_x u_qx(kk,ll) + q_y u_qy(kk,ll)),
 *   q_x = qx_min + (ii-1) + (k-1)/n_row, kk = mod(n_row frac(qx_min) + k, n_row) (0 -> n_row),
 * then the job's species weights, mask and window norm into cs(t, Q) (pixels beyond the zones:
 * 0).  plane 1 = (hk0): b = (b1, b2); plane 2 = (hhl): k from c1 + c2, l = c3,
 * d_x = (d1 + d2 + 2)/sqrt 2, d_y = d3 + 1, b = (b1 + b2, b3).  CELL input on a Q plane with
 * n_row(1) = n_row(2) (= n_row(3) on (hhl)); cell indices set first.  at_base: host
 * float[n_species][3] (the frame header's basis positions).  Asynchronous on the job's stream. */
int mpsq_job_transform_onephonon(mpsq_job* job, int32_t first, int32_t count, int32_t plane,
                                 int32_t n_bz, float qx_min, float qy_min, const float* at_base);

/* Synchronise the job's stream. */
int mpsq_job_sync(mpsq_job* job);

/* Q slab of a job created with q_slab > 0 (no reference counterpart: the reference keeps the
 * whole store, code/src/mp_sqom56.f90:963): kz planes [z0, z0 + min(q_slab, n_qz - z0)).  The
 * next transforms store the amplitudes of those planes only, and the maps (total S(Q), E=const,
 * Gaussian spectrum, I(Q,t), dispersion cuts with slab-local indices) cover the slab, their
 * outputs holding n_qx n_qy (planes of the slab) values with Q index x fastest from plane z0.
 * Asynchronous (host state only); the radial histogram needs the whole store. */
int mpsq_job_set_q_slab(mpsq_job* job, int64_t z0);

/* Run-time choices of a job (no reference counterpart; FINUFFT's opts play this role).  Any
 * change drops the job's captured graphs.
 *   MPSQ_OPT_GRAPH  0 (default): every transform call issues its kernels on the job's stream;
 *                   1: the frame loop of a call is captured once per (first, count) as a CUDA
 *                   graph and replayed with one graph launch.
 *   MPSQ_OPT_SPREAD 0 (default): tensor-core spreading of packed real species pairs;
 *                   1: the CUDA-core FP32 spreading kernel.
 *   MPSQ_OPT_XROWS  rows per CTA of the pruned X pass, 4 or 8 (default).
 *   MPSQ_OPT_LANES  frame lanes used when the job has a second one, 1 or 2 (default).
 *   MPSQ_OPT_ZSLAB  0 (default): spreading, then passes X and Y over whole fine grids;
 *                   a multiple of 16: spreading and passes X and Y run slab by slab of that
 *                   many fine-grid planes over one slab-sized region, which stays in L2
 *                   (FP32 volumes on the pruned transform with tensor-core pair spreading;
 *                   ignored otherwise).
 *   MPSQ_OPT_REPRODUCIBLE  0 (default): records are accumulated within a tile in the order
 *                   the binning's atomics left them, so repeated runs agree to FP32 rounding;
 *                   1: the tensor-core spreading orders each tile's records by content first,
 *                   so that every run, schedule (graph, lanes, z-slabs, other jobs on the GPU)
 *                   and job instance gives bit-identical results (FP32 volumes with packed
 *                   pairs; about 20 % more spreading time, 8 % more per frame). */
#define MPSQ_OPT_GRAPH   1
#define MPSQ_OPT_SPREAD  2
#define MPSQ_OPT_XROWS   3
#define MPSQ_OPT_LANES   4
#define MPSQ_OPT_ZSLAB   5
#define MPSQ_OPT_REPRODUCIBLE 6
int mpsq_job_set_option(mpsq_job* job, int option, int value);
int mpsq_job_get_option(const mpsq_job* job, int option, int* value);

/* Autotuner (no reference counterpart): times mpsq_job_transform(job, first, count) under
 * every combination of the choices above that applies to the job (graph replay, spreading
 * kernel, X-pass rows, frame lanes, z-slab pipeline at 64 planes or none; three calls each,
 * the first untimed), keeps the fastest and sets it on the job.  With a cache_path, a choice
 * recorded there for the same job shape (precision, fine grid, width, grids, packing, pruned
 * transform, lanes) and SM count is taken without timing, and a new choice is appended.
 * choice[4] (optional) returns {graph, spread, xrows, lanes} (the z-slab choice:
 * mpsq_job_get_option); best_ms (optional) the time of one call.  The timed calls rewrite the
 * amplitudes of the same frames. */
int mpsq_job_autotune(mpsq_job* job, int32_t first, int32_t count, const char* cache_path,
                      int* choice, double* best_ms);

/* How a job runs (for reports and tests; no reference counterpart, FINUFFT's plan fields):
 * spreading width, fine-grid lengths [3], number of fine grids per frame (species pairs share
 * one), 1 when the fine-grid transform takes the pruned three-pass kernels (0: cuFFT + separate
 * deconvolution), number of frame lanes (1 or 2).  Any output pointer may be NULL. */
int mpsq_job_info(const mpsq_job* job, int* width, int64_t* fine_grid, int* n_grids, int* pruned,
                  int* lanes);

/* Stage timing with CUDA events on the job's stream.  enable != 0 makes mpsq_job_transform
 * record events around each stage of every frame (and wait for each frame); the accumulated
 * milliseconds of [bin, spread, fft, deconv] and the number of frames timed are returned by
 * mpsq_job_stage_ms (reset != 0 clears them). */
int mpsq_job_profile(mpsq_job* job, int enable);
int mpsq_job_stage_ms(mpsq_job* job, double* ms4, int64_t* frames, int reset);

/* ---- allocation-free 2D type-1 transform -------------------------------------------
 * No counterpart in the reference: an extra entry point of this library for callers that
 * cannot allocate device memory during the call — hosts whose device memory is owned by their
 * own pool under a fixed budget, plug-in hosts that forbid allocation inside a call.  Same
 * transform and mode order as finufft2d1 (FP64), but every array is a DEVICE pointer and all
 * scratch (fine grid, bins, point records, deconvolution factors) lives in a 16 MiB static
 * device array that each GPU loading the library keeps until process exit; it calls no
 * allocator and copies nothing from host memory.  Limits: nj <= 65536 points, ms, mt <= 256
 * modes; larger sizes return MPSQ_ERR_ARG before anything is launched.  Synchronous on
 * `stream` (a cudaStream_t, NULL = default): it returns after reading the device error flag.
 * The first call on a device looks up the static array's address (once per device, with that
 * device current), so make that first call before any stream capture.  Every call reuses the
 * same array, which keeps the previous call's contents (the call clears what must start at
 * zero); calls that overlap on the GPU (other host threads, other streams) race on it and
 * must be serialised by the caller. */
int mpsq_nufft2d1_noalloc(int64_t nj, const double* x, const double* y, const double* c,
                          int iflag, double eps, int64_t ms, int64_t mt, double* fk,
                          void* stream);

/* ---- misc ----------------------------------------------------------------------------- */
const char* mpsq_last_error(void);
/* Library version string. */
const char* mpsq_version(void);
/* Number of kernel launches issued by this library in this process (for reports). */
int64_t mpsq_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* MPSQ_H */
