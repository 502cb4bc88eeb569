! ISO_C_BINDING interface of libimsrg_gb300.so (the C ABI of include/imsrg_gb300.h) for the
! Fortran host of EOM-IMSRG.  Same binding pattern as the reference's zlib module
! (src/gzipmod.f90:5-41): one interface block per C entry point, handles as type(c_ptr),
! scalars by value, arrays and out-arguments by reference.  Every function returns the
! library's status (IMSRG_OK = 0); imsrg_last_error gives the message.
!
! This module depends on nothing of the reference and can be compiled on its own;
! imsrg_gpu_sqop.f90 adds the helpers that move the reference's type(sq_op) across.
! Link: -L<repo>/eom-imsrg_gb300/lib -limsrg_gb300 -Wl,-rpath,<repo>/eom-imsrg_gb300/lib
module imsrg_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int32_t), parameter :: IMSRG_OK = 0, IMSRG_ERR_INVALID_ARGUMENT = 1, IMSRG_ERR_CUDA = 2, &
       IMSRG_ERR_OUT_OF_MEMORY = 3, IMSRG_ERR_NOT_CONVERGED = 4, IMSRG_ERR_MISMATCH = 5, &
       IMSRG_ERR_UNSUPPORTED = 6, IMSRG_ERR_TIMEOUT = 7
  integer(c_int32_t), parameter :: IMSRG_PREC_FP64 = 0, IMSRG_PREC_BF16X3 = 1, IMSRG_PREC_BF16X6 = 2
  integer(c_int32_t), parameter :: IMSRG_COMM_E0 = 1

  ! the fields of type(spd) the engine needs (src/basic_IMSRG.f90:25-37); the arrays are
  ! copied by imsrg_ctx_create and need to live only for that call
  type, bind(C) :: imsrg_basis
     integer(c_int32_t) :: norbits
     type(c_ptr) :: nn, ll, jj, itzp, con
     integer(c_int32_t) :: eMax, lMax
     real(c_double) :: hw
     integer(c_int32_t) :: Aprot, Aneut
  end type imsrg_basis

  type, bind(C) :: imsrg_step_info
     real(c_double) :: E0, mbpt2
     integer(c_int32_t) :: magnus_terms, bch_terms, bch_converged, graph_rebuilt
  end type imsrg_step_info

  interface
     ! ---- context and operators
     function imsrg_ctx_create(basis, device, ctx) bind(C, name='imsrg_ctx_create')
       import :: c_int32_t, c_ptr, imsrg_basis
       type(imsrg_basis), intent(in) :: basis
       integer(c_int32_t), value :: device
       type(c_ptr) :: ctx
       integer(c_int32_t) :: imsrg_ctx_create
     end function imsrg_ctx_create

     function imsrg_ctx_destroy(ctx) bind(C, name='imsrg_ctx_destroy')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int32_t) :: imsrg_ctx_destroy
     end function imsrg_ctx_destroy

     function imsrg_last_error(ctx) bind(C, name='imsrg_last_error')
       import :: c_ptr
       type(c_ptr), value :: ctx
       type(c_ptr) :: imsrg_last_error   ! const char*, NUL-terminated
     end function imsrg_last_error

     function imsrg_set_precision(ctx, mode) bind(C, name='imsrg_set_precision')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: mode
       integer(c_int32_t) :: imsrg_set_precision
     end function imsrg_set_precision

     function imsrg_synchronize(ctx) bind(C, name='imsrg_synchronize')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int32_t) :: imsrg_synchronize
     end function imsrg_synchronize

     function imsrg_op_create(ctx, herm, op) bind(C, name='imsrg_op_create')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: herm
       type(c_ptr) :: op
       integer(c_int32_t) :: imsrg_op_create
     end function imsrg_op_create

     function imsrg_op_destroy(ctx, op) bind(C, name='imsrg_op_destroy')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, op
       integer(c_int32_t) :: imsrg_op_destroy
     end function imsrg_op_destroy

     function imsrg_op_set_herm(ctx, op, herm) bind(C, name='imsrg_op_set_herm')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, op
       integer(c_int32_t), value :: herm
       integer(c_int32_t) :: imsrg_op_set_herm
     end function imsrg_op_set_herm

     ! gam(q*6+g+1) = c_loc(op%mat(q+1)%gam(g+1)%X), c_null_ptr for empty arrays
     function imsrg_op_upload(ctx, op, gam, fhh, fph, fpp, E0) bind(C, name='imsrg_op_upload')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, op
       type(c_ptr), intent(in) :: gam(*)
       real(c_double), intent(in) :: fhh(*), fph(*), fpp(*)
       real(c_double), value :: E0
       integer(c_int32_t) :: imsrg_op_upload
     end function imsrg_op_upload

     function imsrg_op_download(ctx, op, gam, fhh, fph, fpp, E0) bind(C, name='imsrg_op_download')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, op
       type(c_ptr), intent(in) :: gam(*)
       real(c_double) :: fhh(*), fph(*), fpp(*), E0
       integer(c_int32_t) :: imsrg_op_download
     end function imsrg_op_download

     ! the whole operator as one array in the engine's order (vectorize-like)
     function imsrg_op_upload_slab(ctx, op, slab) bind(C, name='imsrg_op_upload_slab')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, op
       real(c_double), intent(in) :: slab(*)
       integer(c_int32_t) :: imsrg_op_upload_slab
     end function imsrg_op_upload_slab

     function imsrg_op_download_slab(ctx, op, slab) bind(C, name='imsrg_op_download_slab')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, op
       real(c_double) :: slab(*)
       integer(c_int32_t) :: imsrg_op_download_slab
     end function imsrg_op_download_slab

     ! ---- operator algebra (src/basic_IMSRG.f90)
     function imsrg_copy_sq_op(ctx, H, op) bind(C, name='imsrg_copy_sq_op')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, H, op
       integer(c_int32_t) :: imsrg_copy_sq_op
     end function imsrg_copy_sq_op

     function imsrg_add_sq_op(ctx, A, ax, B, bx, C) bind(C, name='imsrg_add_sq_op')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, A, B, C
       real(c_double), value :: ax, bx
       integer(c_int32_t) :: imsrg_add_sq_op
     end function imsrg_add_sq_op

     function imsrg_mat_frob_norm(ctx, op, out) bind(C, name='imsrg_mat_frob_norm')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, op
       real(c_double) :: out
       integer(c_int32_t) :: imsrg_mat_frob_norm
     end function imsrg_mat_frob_norm

     function imsrg_mbpt2(ctx, H, out) bind(C, name='imsrg_mbpt2')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, H
       real(c_double) :: out
       integer(c_int32_t) :: imsrg_mbpt2
     end function imsrg_mbpt2

     ! ---- the commutator (src/commutators.f90, call order of src/IMSRG_MAGNUS.f90:207-219)
     function imsrg_commutator(ctx, L, R, RES, flags) bind(C, name='imsrg_commutator')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, L, R, RES
       integer(c_int32_t), value :: flags
       integer(c_int32_t) :: imsrg_commutator
     end function imsrg_commutator

     function imsrg_commutator_110(ctx, L, R, out) bind(C, name='imsrg_commutator_110')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, L, R
       real(c_double) :: out
       integer(c_int32_t) :: imsrg_commutator_110
     end function imsrg_commutator_110

     function imsrg_commutator_220(ctx, L, R, out) bind(C, name='imsrg_commutator_220')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, L, R
       real(c_double) :: out
       integer(c_int32_t) :: imsrg_commutator_220
     end function imsrg_commutator_220

     function imsrg_commutator_111(ctx, L, R, RES) bind(C, name='imsrg_commutator_111')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, L, R, RES
       integer(c_int32_t) :: imsrg_commutator_111
     end function imsrg_commutator_111

     function imsrg_commutator_121(ctx, L, R, RES) bind(C, name='imsrg_commutator_121')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, L, R, RES
       integer(c_int32_t) :: imsrg_commutator_121
     end function imsrg_commutator_121

     function imsrg_commutator_122(ctx, L, R, RES) bind(C, name='imsrg_commutator_122')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, L, R, RES
       integer(c_int32_t) :: imsrg_commutator_122
     end function imsrg_commutator_122

     function imsrg_commutator_222_pp_hh(ctx, L, R, RES, w1, w2) bind(C, name='imsrg_commutator_222_pp_hh')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, L, R, RES, w1, w2
       integer(c_int32_t) :: imsrg_commutator_222_pp_hh
     end function imsrg_commutator_222_pp_hh

     function imsrg_commutator_221(ctx, L, R, RES, w1, w2) bind(C, name='imsrg_commutator_221')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, L, R, RES, w1, w2
       integer(c_int32_t) :: imsrg_commutator_221
     end function imsrg_commutator_221

     function imsrg_cc_create(ctx, kind, cc) bind(C, name='imsrg_cc_create')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: kind
       type(c_ptr) :: cc
       integer(c_int32_t) :: imsrg_cc_create
     end function imsrg_cc_create

     function imsrg_calculate_cross_coupled(ctx, HS, CCME) bind(C, name='imsrg_calculate_cross_coupled')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, HS, CCME
       integer(c_int32_t) :: imsrg_calculate_cross_coupled
     end function imsrg_calculate_cross_coupled

     function imsrg_commutator_222_ph(ctx, LCC, RCC, RES, WCC) bind(C, name='imsrg_commutator_222_ph')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, LCC, RCC, RES, WCC
       integer(c_int32_t) :: imsrg_commutator_222_ph
     end function imsrg_commutator_222_ph

     ! ---- generator and flow (src/generators.f90, src/IMSRG_MAGNUS.f90)
     function imsrg_build_gs_white(ctx, H, ETA) bind(C, name='imsrg_build_gs_white')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, H, ETA
       integer(c_int32_t) :: imsrg_build_gs_white
     end function imsrg_build_gs_white

     function imsrg_magnus_expand(ctx, DG, G, used) bind(C, name='imsrg_magnus_expand')
       import :: c_int32_t, c_ptr
       type(c_ptr), value :: ctx, DG, G
       integer(c_int32_t) :: used
       integer(c_int32_t) :: imsrg_magnus_expand
     end function imsrg_magnus_expand

     function imsrg_euler_step(ctx, G, DG, s, stp) bind(C, name='imsrg_euler_step')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, G, DG
       real(c_double) :: s
       real(c_double), value :: stp
       integer(c_int32_t) :: imsrg_euler_step
     end function imsrg_euler_step

     function imsrg_bch_expand(ctx, HS, G, H, max_terms, conv, used) bind(C, name='imsrg_bch_expand')
       import :: c_int32_t, c_ptr, c_double
       type(c_ptr), value :: ctx, HS, G, H
       integer(c_int32_t), value :: max_terms
       real(c_double), value :: conv
       integer(c_int32_t) :: used
       integer(c_int32_t) :: imsrg_bch_expand
     end function imsrg_bch_expand

     function imsrg_magnus_step(ctx, HS, G, DG, H, ds, max_terms, conv, use_graph, info) &
          bind(C, name='imsrg_magnus_step')
       import :: c_int32_t, c_ptr, c_double, imsrg_step_info
       type(c_ptr), value :: ctx, HS, G, DG, H
       real(c_double), value :: ds, conv
       integer(c_int32_t), value :: max_terms, use_graph
       type(imsrg_step_info) :: info
       integer(c_int32_t) :: imsrg_magnus_step
     end function imsrg_magnus_step

     ! the same step with the flow state in pinned host slabs (inputs omega, eta, H; outputs
     ! H(s), omega, eta); some copies overlap the step inside the captured graph
     function imsrg_magnus_step_host(ctx, HS, G, DG, H, hs_host, g_host, dg_host, h_host, ds, max_terms, conv, &
          use_graph, info) bind(C, name='imsrg_magnus_step_host')
       import :: c_int32_t, c_ptr, c_double, imsrg_step_info
       type(c_ptr), value :: ctx, HS, G, DG, H, hs_host, g_host, dg_host, h_host
       real(c_double), value :: ds, conv
       integer(c_int32_t), value :: max_terms, use_graph
       type(imsrg_step_info) :: info
       integer(c_int32_t) :: imsrg_magnus_step_host
     end function imsrg_magnus_step_host
  end interface

contains

  ! the C string of imsrg_last_error as a Fortran string
  function imsrg_error_text(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: chars(:)
    integer :: n
    interface
       function strlen(s) bind(C, name='strlen')
         import :: c_ptr, c_size_t
         type(c_ptr), value :: s
         integer(c_size_t) :: strlen
       end function strlen
    end interface
    type(c_ptr) :: p
    p = imsrg_last_error(ctx)
    n = int(strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: msg)
    msg = transfer(chars(1:n), msg)
  end function imsrg_error_text

  ! stop with the library's message on a failed call (the reference's own error style)
  subroutine imsrg_check(ctx, st, where)
    type(c_ptr), intent(in) :: ctx
    integer(c_int32_t), intent(in) :: st
    character(len=*), intent(in) :: where
    if (st /= IMSRG_OK) then
       write(*, '(A,A,A,I0,A,A)') 'imsrg_gpu: ', where, ' failed with status ', st, ': ', imsrg_error_text(ctx)
       stop 1
    end if
  end subroutine imsrg_check

end module imsrg_gpu
