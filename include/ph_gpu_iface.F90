! ISO_C_BINDING interface of libphantom_gb300 (include/phantom_gb300.h) for
! Phantom's Fortran step loop: the module a maintainer adds to src/main so
! that derivs (src/main/deriv.f90:37-232) can call the GPU path in place of
! maketree / densityiterate / force. Every entry point of the C header has a
! declaration here; array arguments keep the reference's layouts
! (part.F90:47-391): xyzh(4,*), vxyzu(maxvxyzu,*), Bevol(4,*), fxyzu(maxvxyzu,*)
! and dBevol(4,*) double, gradh(2,*), divcurlv(*), divcurlB(4,*), divBsymm(*)
! and poten(*) float.
module ph_gpu_iface
 use, intrinsic :: iso_c_binding
 implicit none
 type, bind(c) :: ph_params
    integer(c_int32_t) :: periodic, mhd, gravity, isothermal, ieos
    integer(c_int32_t) :: ipdv_heating, ishock_heating, iresistive_heating
    integer(c_int32_t) :: precision, minpart   ! minpart 0: the reference's 10
    real(c_double)     :: xmin, xmax, ymin, ymax, zmin, zmax
    real(c_double)     :: hfact, tolh, massoftype
    real(c_double)     :: alpha, alphau, alphaB, beta
    real(c_double)     :: gamma, polyk
    real(c_double)     :: C_cour, C_force, tolv, dtmax
    real(c_double)     :: psidecayfac, overcleanfac
    real(c_double)     :: tree_accuracy
    integer(c_int64_t) :: maxp
    real(c_double)     :: alphamax               ! shock_capturing alphamax (0: 1.0)
    integer(c_int32_t) :: nalpha, ind_timesteps  ! nalpha: 0 with CONST_AV, 3 otherwise (config.F90:158-162);
                                                 ! ind_timesteps: 1 with IND_TIMESTEPS
    integer(c_int32_t) :: maxvxyzu               ! config.F90:50-53: set to maxvxyzu (3 with ISOTHERMAL),
                                                 ! so vxyzu and fxyzu pass as allocated in part.F90
    integer(c_int32_t) :: curlv                  ! config.F90:166,384: 1 when curlv (ndivcurlv = 4), so
                                                 ! divcurlv passes as allocated in part.F90
 end type ph_params
 type, bind(c) :: ph_tune
    integer(c_int32_t) :: minpart, dens_warps, force_warps, walk_warps
    real(c_double)     :: ms_before, ms_after
    integer(c_int32_t) :: force_sym   ! 1: FP64 force pairs evaluated once for both particles
 end type ph_tune
 interface
  integer(c_int) function ph_init(p, maxp, ctx) bind(c, name="ph_init")
    import; type(ph_params), intent(in) :: p; integer(c_int64_t), value :: maxp; type(c_ptr) :: ctx
  end function
  integer(c_int) function ph_upload(ctx, npart, xyzh, vxyzu, Bevol) bind(c, name="ph_upload")
    import; type(c_ptr), value :: ctx; integer(c_int64_t), value :: npart
    real(c_double), intent(in) :: xyzh(4,*), vxyzu(*), Bevol(4,*)   ! vxyzu(maxvxyzu,*)
  end function
  integer(c_int) function ph_build_tree(ctx, xyzh, inodeparts, ncells) bind(c, name="ph_build_tree")
    import; type(c_ptr), value :: ctx; real(c_double) :: xyzh(4,*)
    integer(c_int32_t) :: inodeparts(*); integer(c_int64_t) :: ncells
  end function
  integer(c_int) function ph_density(ctx, icall, xyzh, gradh, divcurlv, divcurlB, nneigh, hash, stats) &
       bind(c, name="ph_density")
    import; type(c_ptr), value :: ctx; integer(c_int), value :: icall
    real(c_double) :: xyzh(4,*); real(c_float) :: gradh(2,*), divcurlv(*), divcurlB(4,*)
    type(c_ptr), value :: nneigh, hash, stats
  end function
  integer(c_int) function ph_force(ctx, icall, dt, fxyzu, dBevol, divcurlv, divBsymm, poten, dtcourant, dtforce) &
       bind(c, name="ph_force")
    import; type(c_ptr), value :: ctx; integer(c_int), value :: icall; real(c_double), value :: dt
    real(c_double) :: fxyzu(*), dBevol(4,*); real(c_float) :: divcurlv(*), divBsymm(*), poten(*)
    real(c_double) :: dtcourant, dtforce
  end function
  integer(c_int) function ph_step(ctx, t, dtsph, dtnew, its, dterr) bind(c, name="ph_step")
    import; type(c_ptr), value :: ctx; real(c_double), value :: t, dtsph
    real(c_double) :: dtnew, dterr; integer(c_int32_t) :: its
  end function
  integer(c_int) function ph_adjoint(ctx, w_fxyzu, g_xyzh, g_vxyzu, g_Bevol) bind(c, name="ph_adjoint")
    import; type(c_ptr), value :: ctx
    real(c_double), intent(in) :: w_fxyzu(*); real(c_double) :: g_xyzh(4,*), g_vxyzu(*)
    type(c_ptr), value :: g_Bevol
  end function
  integer(c_int) function ph_adjoint_full(ctx, w_fxyzu, w_dBevol, g_xyzh, g_vxyzu, g_Bevol) &
       bind(c, name="ph_adjoint_full")
    import; type(c_ptr), value :: ctx
    real(c_double), intent(in) :: w_fxyzu(*); real(c_double) :: g_xyzh(4,*), g_vxyzu(*)
    type(c_ptr), value :: w_dBevol, g_Bevol   ! c_loc of w_dBevol(4,*), g_Bevol(4,*) with MHD, else c_null_ptr
  end function
  integer(c_int) function ph_rollout_adjoint(ctx, nsteps, dts, ckpt, w_fxyzu, loss, g_xyzh, g_vxyzu) &
       bind(c, name="ph_rollout_adjoint")
    import; type(c_ptr), value :: ctx; integer(c_int32_t), value :: nsteps, ckpt
    real(c_double), intent(in) :: dts(*), w_fxyzu(*); real(c_double) :: loss, g_xyzh(4,*), g_vxyzu(*)
  end function
  integer(c_int) function ph_rollout_adjoint_full(ctx, nsteps, dts, ckpt, w_fxyzu, w_dBevol, loss, g_xyzh, &
       g_vxyzu, g_Bevol) bind(c, name="ph_rollout_adjoint_full")
    import; type(c_ptr), value :: ctx; integer(c_int32_t), value :: nsteps, ckpt
    real(c_double), intent(in) :: dts(*), w_fxyzu(*); real(c_double) :: loss, g_xyzh(4,*), g_vxyzu(*)
    type(c_ptr), value :: w_dBevol, g_Bevol   ! c_loc of (4,*) arrays with MHD, else c_null_ptr
  end function
  integer(c_int) function ph_set_alpha(ctx, alpha) bind(c, name="ph_set_alpha")
    import; type(c_ptr), value :: ctx; real(c_float), intent(in) :: alpha(*)
  end function
  integer(c_int) function ph_get_alpha(ctx, alphaind, dvdx) bind(c, name="ph_get_alpha")
    import; type(c_ptr), value :: ctx; real(c_float) :: alphaind(3,*), dvdx(9,*)
  end function
  integer(c_int) function ph_alpha_initial(ctx) bind(c, name="ph_alpha_initial")
    import; type(c_ptr), value :: ctx
  end function
  integer(c_int) function ph_ind_init(ctx, time) bind(c, name="ph_ind_init")
    import; type(c_ptr), value :: ctx; real(c_double), value :: time
  end function
  integer(c_int) function ph_ind_substep(ctx, time, nactive) bind(c, name="ph_ind_substep")
    import; type(c_ptr), value :: ctx; real(c_double) :: time; integer(c_int64_t) :: nactive
  end function
  integer(c_int) function ph_ind_state(ctx, ibin, twas, counters) bind(c, name="ph_ind_state")
    import; type(c_ptr), value :: ctx; integer(c_int8_t) :: ibin(*); real(c_double) :: twas(*)
    integer(c_int32_t) :: counters(4)
  end function
  integer(c_int) function ph_set_params(ctx, p) bind(c, name="ph_set_params")
    import; type(c_ptr), value :: ctx; type(ph_params), intent(in) :: p
  end function
  subroutine ph_finalize(ctx) bind(c, name="ph_finalize")
    import; type(c_ptr), value :: ctx
  end subroutine
  integer(c_int) function ph_derivs(ctx, icall, dt, dtnew) bind(c, name="ph_derivs")
    import; type(c_ptr), value :: ctx; integer(c_int), value :: icall; real(c_double), value :: dt
    real(c_double) :: dtnew
  end function
  integer(c_int) function ph_download(ctx, xyzh, vxyzu, Bevol) bind(c, name="ph_download")
    import; type(c_ptr), value :: ctx; real(c_double) :: xyzh(4,*), vxyzu(*), Bevol(4,*)
  end function
  integer(c_int) function ph_upload_state(ctx, npart, xyzh, vxyzu, Bevol, fxyzu, dBevol, divcurlv) &
       bind(c, name="ph_upload_state")
    import; type(c_ptr), value :: ctx; integer(c_int64_t), value :: npart
    real(c_double), intent(in) :: xyzh(4,*), vxyzu(*), Bevol(4,*), fxyzu(*), dBevol(4,*)
    real(c_float), intent(in) :: divcurlv(*)
  end function
  integer(c_int) function ph_download_state(ctx, xyzh, vxyzu, Bevol, fxyzu, dBevol, divcurlv) &
       bind(c, name="ph_download_state")
    import; type(c_ptr), value :: ctx
    real(c_double) :: xyzh(4,*), vxyzu(*), Bevol(4,*), fxyzu(*), dBevol(4,*); real(c_float) :: divcurlv(*)
  end function
  integer(c_int) function ph_conservation(ctx, out) bind(c, name="ph_conservation")
    import; type(c_ptr), value :: ctx; real(c_double) :: out(8)
  end function
  integer(c_int) function ph_conservation_noalloc(p, npart, xyzh, vxyzu, fxyzu, Bevol, poten, out, stream) &
       bind(c, name="ph_conservation_noalloc")
    import; type(ph_params), intent(in) :: p; integer(c_int64_t), value :: npart
    type(c_ptr), value :: xyzh, vxyzu, fxyzu, Bevol, poten, out, stream   ! device addresses
  end function
  integer(c_int) function ph_revtree(ctx, xyzh) bind(c, name="ph_revtree")
    import; type(c_ptr), value :: ctx; real(c_double), intent(in) :: xyzh(4,*)
  end function
  integer(c_int) function ph_get_nodes(ctx, nnodes, inoderange, xcen, size, hmax, mass, isleaf) &
       bind(c, name="ph_get_nodes")
    import; type(c_ptr), value :: ctx; integer(c_int64_t) :: nnodes
    integer(c_int32_t) :: inoderange(2,*), isleaf(*); real(c_double) :: xcen(3,*), size(*), hmax(*), mass(*)
  end function
  integer(c_int) function ph_last_timings(ctx, ms8) bind(c, name="ph_last_timings")
    import; type(c_ptr), value :: ctx; real(c_double) :: ms8(8)
  end function
  integer(c_int) function ph_work_counters(ctx, out4) bind(c, name="ph_work_counters")
    import; type(c_ptr), value :: ctx; integer(c_int64_t) :: out4(4)
  end function
  integer(c_int64_t) function ph_kernel_launches(ctx) bind(c, name="ph_kernel_launches")
    import; type(c_ptr), value :: ctx
  end function
  integer(c_int) function ph_autotune(ctx, flags, t) bind(c, name="ph_autotune")
    import; type(c_ptr), value :: ctx; integer(c_int), value :: flags; type(ph_tune) :: t
  end function
  integer(c_int) function ph_get_tune(ctx, t) bind(c, name="ph_get_tune")
    import; type(c_ptr), value :: ctx; type(ph_tune) :: t
  end function
  integer(c_int) function ph_set_tune(ctx, t) bind(c, name="ph_set_tune")
    import; type(c_ptr), value :: ctx; type(ph_tune), intent(in) :: t
  end function
  type(c_ptr) function ph_strerror(code) bind(c, name="ph_strerror")
    import; integer(c_int), value :: code
  end function
 end interface
end module ph_gpu_iface
