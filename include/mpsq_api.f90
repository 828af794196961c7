! ISO_C_BINDING interface to the batched job API of libmpsq (include/mpsq.h), for a Fortran
! host such as mp_sqom / mp_sql.  The derived type mpsq_job_desc_t has the member order and
! types of the C struct mpsq_job_desc; C arrays [k][b] appear transposed, as (b, k).
! Link: -L<path to mp_tools_gb300/_build> -lmpsq
module mpsq_api
  use iso_c_binding
  implicit none
  private

  integer(c_int), parameter, public :: MPSQ_MAX_SPECIES = 16
  integer(c_int), parameter, public :: MPSQ_FP32 = 0, MPSQ_FP64 = 1
  integer(c_int), parameter, public :: MPSQ_CELL = 0, MPSQ_BULK = 1
  integer(c_int), parameter, public :: MPSQ_WEIGHT_UNIT = 1, MPSQ_WEIGHT_NEUTRON = 2, &
                                       MPSQ_WEIGHT_XRAY = 3
  ! run-time choices (mpsq_job_set_option / mpsq_job_get_option)
  integer(c_int), parameter, public :: MPSQ_OPT_GRAPH = 1, MPSQ_OPT_SPREAD = 2, &
                                       MPSQ_OPT_XROWS = 3, MPSQ_OPT_LANES = 4, &
                                       MPSQ_OPT_ZSLAB = 5, MPSQ_OPT_REPRODUCIBLE = 6

  type, bind(C), public :: mpsq_job_desc_t
    integer(c_int32_t) :: ndim
    integer(c_int32_t) :: precision
    real(c_double)     :: eps
    integer(c_int64_t) :: n_modes(3)
    integer(c_int32_t) :: input_method
    integer(c_int32_t) :: phase_rounding
    real(c_double)     :: axis(3, 3)            ! axis(b, k) = component b of unit vector e_k
    real(c_double)     :: tpe(3)
    real(c_double)     :: centre(3)
    integer(c_int32_t) :: use_range
    real(c_double)     :: pos_min(3)
    real(c_double)     :: pos_max(3)
    real(c_double)     :: eps_x
    integer(c_int32_t) :: bulk_nsuper1
    integer(c_int32_t) :: n_row(3)
    real(c_double)     :: q_center(3)
    integer(c_int32_t) :: spatial_window
    integer(c_int32_t) :: n_species
    integer(c_int64_t) :: species_offset(17)    ! MPSQ_MAX_SPECIES + 1
    integer(c_int32_t) :: mask(16)
    integer(c_int32_t) :: weight_mode
    real(c_double)     :: b_coh(16)
    real(c_double)     :: xff(9, 16)            ! xff(i, s): a1 b1 a2 b2 a3 b3 a4 b4 c of species s
    integer(c_int32_t) :: ff_convention
    real(c_double)     :: qphys_origin(3)
    real(c_double)     :: qphys_step(3, 3)      ! qphys_step(b, k)
    real(c_double)     :: qphys_extra_sq
    integer(c_int64_t) :: n_atoms_frame
    integer(c_int32_t) :: n_frames
    integer(c_int32_t) :: store_species
    integer(c_int32_t) :: no_pack
    integer(c_int32_t) :: no_pruned_fft
    integer(c_int32_t) :: stream_ordered
    integer(c_int64_t) :: q_slab
  end type

  public :: mpsq_job_create, mpsq_job_destroy, mpsq_job_estimate_bytes, mpsq_job_set_frames, &
            mpsq_job_set_cell_index, mpsq_job_transform, mpsq_job_sq_total, &
            mpsq_job_sqw_econst, mpsq_job_sqw_dispersion, mpsq_job_iqt, mpsq_job_sync, &
            mpsq_speckle_filter, mpsq_job_transform_onephonon, mpsq_last_error

  interface
    integer(c_int) function mpsq_job_create(desc, stream, job) bind(C, name="mpsq_job_create")
      import :: c_int, c_ptr, mpsq_job_desc_t
      type(mpsq_job_desc_t), intent(in) :: desc
      type(c_ptr), value :: stream                 ! cudaStream_t, c_null_ptr = default stream
      type(c_ptr), intent(out) :: job
    end function

    integer(c_int) function mpsq_job_destroy(job) bind(C, name="mpsq_job_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: job
    end function

    integer(c_int) function mpsq_job_estimate_bytes(desc, bytes) &
        bind(C, name="mpsq_job_estimate_bytes")
      import :: c_int, c_int64_t, mpsq_job_desc_t
      type(mpsq_job_desc_t), intent(in) :: desc
      integer(c_int64_t), intent(out) :: bytes
    end function

    integer(c_int) function mpsq_job_set_frames(job, pos, first, count, host) &
        bind(C, name="mpsq_job_set_frames")
      import :: c_int, c_int32_t, c_ptr, c_float
      type(c_ptr), value :: job
      real(c_float), intent(in) :: pos(*)          ! at_pos(4, n_atoms, count), frame-major
      integer(c_int32_t), value :: first, count
      integer(c_int), value :: host
    end function

    integer(c_int) function mpsq_job_set_cell_index(job, at_ind, host) &
        bind(C, name="mpsq_job_set_cell_index")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: job
      integer(c_int32_t), intent(in) :: at_ind(*)  ! at_ind(4, n_atoms)
      integer(c_int), value :: host
    end function

    integer(c_int) function mpsq_job_transform(job, first, count) bind(C, name="mpsq_job_transform")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: job
      integer(c_int32_t), value :: first, count
    end function

    integer(c_int) function mpsq_job_sq_total(job, norm2, out, host) bind(C, name="mpsq_job_sq_total")
      import :: c_int, c_ptr, c_double, c_float
      type(c_ptr), value :: job
      real(c_double), value :: norm2
      real(c_float), intent(out) :: out(*)
      integer(c_int), value :: host
    end function

    integer(c_int) function mpsq_job_sqw_econst(job, n_int, t_wind, j_freq, q2_norm, scale, out, &
                                                host) bind(C, name="mpsq_job_sqw_econst")
      import :: c_int, c_int32_t, c_ptr, c_double, c_float
      type(c_ptr), value :: job
      integer(c_int32_t), value :: n_int, j_freq
      real(c_float), intent(in) :: t_wind(*)
      type(c_ptr), value :: q2_norm                 ! real(c_float) array or c_null_ptr
      real(c_double), value :: scale
      real(c_float), intent(out) :: out(*)
      integer(c_int), value :: host
    end function

    integer(c_int) function mpsq_job_sqw_dispersion(job, n_int, t_wind, n_path, q_index, n_freq, &
                                                    q2_norm, scale, out, host) &
        bind(C, name="mpsq_job_sqw_dispersion")
      import :: c_int, c_int32_t, c_int64_t, c_ptr, c_double, c_float
      type(c_ptr), value :: job
      integer(c_int32_t), value :: n_int, n_path, n_freq
      real(c_float), intent(in) :: t_wind(*)
      integer(c_int64_t), intent(in) :: q_index(*)
      type(c_ptr), value :: q2_norm
      real(c_double), value :: scale
      real(c_float), intent(out) :: out(*)
      integer(c_int), value :: host
    end function

    integer(c_int) function mpsq_job_iqt(job, n_int, lag, q2_norm, scale, out, host) &
        bind(C, name="mpsq_job_iqt")
      import :: c_int, c_int32_t, c_ptr, c_double, c_float
      type(c_ptr), value :: job
      integer(c_int32_t), value :: n_int, lag
      type(c_ptr), value :: q2_norm
      real(c_double), value :: scale
      real(c_float), intent(out) :: out(*)
      integer(c_int), value :: host
    end function

    integer(c_int) function mpsq_job_sync(job) bind(C, name="mpsq_job_sync")
      import :: c_int, c_ptr
      type(c_ptr), value :: job
    end function

    integer(c_int) function mpsq_speckle_filter(map, n_fast, n_slow, s_trig, perpendicular, &
                                                post_scale, host, stream) &
        bind(C, name="mpsq_speckle_filter")
      import :: c_int, c_int32_t, c_int64_t, c_ptr, c_float
      real(c_float), intent(inout) :: map(*)        ! cs_plot(n_fast, n_slow)
      integer(c_int64_t), value :: n_fast, n_slow
      real(c_float), value :: s_trig, post_scale
      integer(c_int32_t), value :: perpendicular, host
      type(c_ptr), value :: stream
    end function

    integer(c_int) function mpsq_job_transform_onephonon(job, first, count, plane, n_bz, qx_min, &
                                                         qy_min, at_base) &
        bind(C, name="mpsq_job_transform_onephonon")
      import :: c_int, c_int32_t, c_ptr, c_float
      type(c_ptr), value :: job
      integer(c_int32_t), value :: first, count, plane, n_bz
      real(c_float), value :: qx_min, qy_min
      real(c_float), intent(in) :: at_base(*)       ! at_base(3, n_species)
    end function

    integer(c_int) function mpsq_job_set_q_slab(job, z0) bind(C, name="mpsq_job_set_q_slab")
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: job
      integer(c_int64_t), value :: z0
    end function

    integer(c_int) function mpsq_job_set_option(job, option, val) &
        bind(C, name="mpsq_job_set_option")
      import :: c_int, c_ptr
      type(c_ptr), value :: job
      integer(c_int), value :: option, val
    end function

    integer(c_int) function mpsq_job_get_option(job, option, val) &
        bind(C, name="mpsq_job_get_option")
      import :: c_int, c_ptr
      type(c_ptr), value :: job
      integer(c_int), value :: option
      integer(c_int), intent(out) :: val
    end function

    integer(c_int) function mpsq_job_autotune(job, first, count, cache_path, choice, best_ms) &
        bind(C, name="mpsq_job_autotune")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: job
      integer(c_int32_t), value :: first, count
      type(c_ptr), value :: cache_path                ! C string (c_null_char-terminated) or null
      integer(c_int), intent(out) :: choice(4)       ! graph, spread, xrows, lanes
      real(c_double), intent(out) :: best_ms
    end function

    integer(c_int) function mpsq_job_info(job, width, fine_grid, n_grids, pruned, lanes) &
        bind(C, name="mpsq_job_info")
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: job
      integer(c_int), intent(out) :: width, n_grids, pruned, lanes
      integer(c_int64_t), intent(out) :: fine_grid(3)
    end function

    type(c_ptr) function mpsq_last_error() bind(C, name="mpsq_last_error")
      import :: c_ptr
    end function
  end interface
end module mpsq_api
