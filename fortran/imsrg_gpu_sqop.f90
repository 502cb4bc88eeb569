! Helpers that move the reference's own types across the imsrg_gpu binding: a context from
! type(spd) and a reference operator, and type(sq_op) operators to and from device
! operators.  Compiled inside the EOM-IMSRG tree (it uses the module basic_IMSRG of
! src/basic_IMSRG.f90), after imsrg_gpu.f90.
!
! Drop-in use at the call sites of src/IMSRG_MAGNUS.f90:207-219 (one commutator of
! BCH_EXPAND) -- the sq_op arrays stay where they are, the device holds its own copies:
!
!     call gpu_context(jbas, H, ctx)                       ! once per basis
!     call gpu_new_op(ctx, L, dL); call gpu_new_op(ctx, R, dR); call gpu_new_op(ctx, RES, dRES)
!     call gpu_put(ctx, dL, L); call gpu_put(ctx, dR, R)
!     call imsrg_check(ctx, imsrg_commutator(ctx, dL, dR, dRES, IMSRG_COMM_E0), 'commutator')
!     call gpu_get(ctx, dRES, RES)
!
! and the loop body of magnus_decouple (src/IMSRG_MAGNUS.f90:47-110) is one
! imsrg_magnus_step call on device operators.
module imsrg_gpu_sqop
  use, intrinsic :: iso_c_binding
  use basic_IMSRG
  use imsrg_gpu
  implicit none

contains

  ! imsrg_ctx_create from the basis descriptor and the operator's A, eMax, lmax, hw
  ! (read_sp_basis + store_6j + allocate_blocks + allocate_CCMAT on the device)
  subroutine gpu_context(jbas, op, ctx, device)
    type(spd), intent(in) :: jbas
    type(sq_op), intent(in) :: op
    type(c_ptr), intent(out) :: ctx
    integer, intent(in), optional :: device
    integer(c_int32_t), allocatable, target :: nn(:), ll(:), jj(:), tz(:), con(:)
    type(imsrg_basis) :: b
    integer(c_int32_t) :: dev, st
    dev = 0
    if (present(device)) dev = int(device, c_int32_t)
    allocate(nn(jbas%total_orbits), ll(jbas%total_orbits), jj(jbas%total_orbits), &
         tz(jbas%total_orbits), con(jbas%total_orbits))
    nn = int(jbas%nn, c_int32_t); ll = int(jbas%ll, c_int32_t); jj = int(jbas%jj, c_int32_t)
    tz = int(jbas%itzp, c_int32_t); con = int(jbas%con, c_int32_t)
    b%norbits = int(jbas%total_orbits, c_int32_t)
    b%nn = c_loc(nn); b%ll = c_loc(ll); b%jj = c_loc(jj); b%itzp = c_loc(tz); b%con = c_loc(con)
    b%eMax = int(op%eMax, c_int32_t); b%lMax = int(op%lmax, c_int32_t)
    b%hw = real(op%hospace, c_double)
    b%Aprot = int(op%Aprot, c_int32_t); b%Aneut = int(op%Aneut, c_int32_t)
    ctx = c_null_ptr
    st = imsrg_ctx_create(b, dev, ctx)
    if (st /= IMSRG_OK) then
       write(*, '(A,I0)') 'imsrg_gpu: imsrg_ctx_create failed with status ', st
       stop 1
    end if
  end subroutine gpu_context

  ! a device operator with the herm flag of op
  subroutine gpu_new_op(ctx, op, dop)
    type(c_ptr), intent(in) :: ctx
    type(sq_op), intent(in) :: op
    type(c_ptr), intent(out) :: dop
    dop = c_null_ptr
    call imsrg_check(ctx, imsrg_op_create(ctx, int(op%herm, c_int32_t), dop), 'imsrg_op_create')
  end subroutine gpu_new_op

  ! c_loc of every op%mat(q)%gam(g)%X in the order the library expects (q-major, g = 1..6);
  ! empty arrays pass c_null_ptr
  subroutine gam_pointers(op, gam)
    type(sq_op), intent(in), target :: op
    type(c_ptr), intent(out) :: gam(:)
    integer :: q, g
    do q = 1, op%nblocks
       do g = 1, 6
          if (size(op%mat(q)%gam(g)%X) > 0) then
             gam((q - 1) * 6 + g) = c_loc(op%mat(q)%gam(g)%X(1, 1))
          else
             gam((q - 1) * 6 + g) = c_null_ptr
          end if
       end do
    end do
  end subroutine gam_pointers

  ! host sq_op -> device operator (herm flag included)
  subroutine gpu_put(ctx, dop, op)
    type(c_ptr), intent(in) :: ctx, dop
    type(sq_op), intent(in), target :: op
    type(c_ptr), allocatable :: gam(:)
    allocate(gam(6 * op%nblocks))
    call gam_pointers(op, gam)
    call imsrg_check(ctx, imsrg_op_set_herm(ctx, dop, int(op%herm, c_int32_t)), 'imsrg_op_set_herm')
    call imsrg_check(ctx, imsrg_op_upload(ctx, dop, gam, op%fhh, op%fph, op%fpp, real(op%E0, c_double)), &
         'imsrg_op_upload')
  end subroutine gpu_put

  ! device operator -> host sq_op (arrays allocated by allocate_blocks / duplicate_sq_op)
  subroutine gpu_get(ctx, dop, op)
    type(c_ptr), intent(in) :: ctx, dop
    type(sq_op), intent(inout), target :: op
    type(c_ptr), allocatable :: gam(:)
    real(c_double) :: e0
    allocate(gam(6 * op%nblocks))
    call gam_pointers(op, gam)
    call imsrg_check(ctx, imsrg_op_download(ctx, dop, gam, op%fhh, op%fph, op%fpp, e0), 'imsrg_op_download')
    op%E0 = e0
  end subroutine gpu_get

end module imsrg_gpu_sqop
