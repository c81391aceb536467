!> @brief GB300 linear accelerator behind ImsLinearDataType (ISO_C_BINDING)
!!
!! This module sits next to src/Solution/LinearMethods/ImsLinear.f90 and binds
!! the C ABI of libgbims.so (include/gbims.h).  ImsGb300Type keeps the
!! reference's allocate / apply / deallocate contract
!! (imslinear_allocate ImsLinear.f90:111-339, imslinear_ap :617-750,
!! imslinear_da :495-552): the solution still owns AMAT, RHS and X, X is the
!! initial guess on entry and the solution on exit, AMAT and RHS come back
!! unchanged, and ICNVG / IN_ITER keep their meaning.  The per-inner-iteration
!! rows of the ConvergenceSummary (ImsLinearBase.f90:141-197, 431-493) and
!! CACCEL are filled from the device records when NCONV > 1.
!!
!! A negative status from the library becomes a store_error call that stops
!! the run, as the reference's own error paths do (ImsLinear.f90:188-215,
!! ImsLinearBase.f90:827-836); pivot retries (status GBIMS_WARN_PIVOT) are
!! logged and the run goes on (ImsLinearBase.f90:861-863).
!<
module ImsGb300Module
  use iso_c_binding, only: c_int, c_double, c_ptr, c_null_ptr, c_char, &
                           c_associated, c_f_pointer, c_null_char
  use KindModule, only: DP, I4B
  use SimModule, only: store_error
  use ConvergenceSummaryModule, only: ConvergenceSummaryType
  implicit none
  private

  public :: ImsGb300Type
  public :: gbims_settings_t, gbims_summary_t

  integer(c_int), parameter, public :: GBIMS_FP64 = 0, GBIMS_MIXED = 1
  integer(c_int), parameter, public :: GBIMS_OK = 0, GBIMS_WARN_PIVOT = 1

  !> gbims_settings of include/gbims.h, member by member
  type, bind(C) :: gbims_settings_t
    real(c_double) :: dvclose, rclose
    integer(c_int) :: icnvgopt, iter1, ilinmeth, iscl, iord, north
    real(c_double) :: relax
    integer(c_int) :: level
    real(c_double) :: droptol
    integer(c_int) :: precision, index_base, nlay, nrow, ncol
  end type gbims_settings_t

  !> gbims_summary of include/gbims.h, member by member
  type, bind(C) :: gbims_summary_t
    integer(c_int) :: iter_cnt, icnvg, pivot_retries, exit_reason
    real(c_double) :: dvmax
    integer(c_int) :: locdv
    real(c_double) :: rmax
    integer(c_int) :: locr
    real(c_double) :: l2norm0, l2norm, solve_ms
    integer(c_int) :: refinements, structured
  end type gbims_summary_t

  interface
    integer(c_int) function gbims_create(s, neq, nja, ia, ja, h) &
      bind(C, name='gbims_create')
      import :: c_int, c_ptr, gbims_settings_t
      type(gbims_settings_t), intent(in) :: s
      integer(c_int), value :: neq, nja
      integer(c_int), intent(in) :: ia(*), ja(*)
      type(c_ptr), intent(out) :: h
    end function gbims_create
    integer(c_int) function gbims_apply(h, amat, rhs, x, kstp, kiter, icnvg, &
                                        in_iter, summ) &
      bind(C, name='gbims_apply')
      import :: c_int, c_double, c_ptr, gbims_summary_t
      type(c_ptr), value :: h
      real(c_double), intent(inout) :: amat(*), rhs(*), x(*)
      integer(c_int), value :: kstp, kiter
      integer(c_int), intent(out) :: icnvg, in_iter
      type(gbims_summary_t), intent(out) :: summ
    end function gbims_apply
    integer(c_int) function gbims_destroy(h) bind(C, name='gbims_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function gbims_destroy
    type(c_ptr) function gbims_last_error(h) bind(C, name='gbims_last_error')
      import :: c_ptr
      type(c_ptr), value :: h
    end function gbims_last_error
    integer(c_int) function gbims_set_inner_records(h, nconv, convnmod, &
                                                    convmodstart) &
      bind(C, name='gbims_set_inner_records')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nconv, convnmod
      integer(c_int), intent(in) :: convmodstart(*)
    end function gbims_set_inner_records
    integer(c_int) function gbims_get_inner_records(h, cap, nrec, itinner, &
                                                    alpha, omega, locdv, &
                                                    dvmax, locr, rmax) &
      bind(C, name='gbims_get_inner_records')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: cap
      integer(c_int), intent(out) :: nrec
      integer(c_int), intent(out) :: itinner(*), locdv(*), locr(*)
      real(c_double), intent(out) :: alpha(*), omega(*), dvmax(*), rmax(*)
    end function gbims_get_inner_records
    ! a DIS grid reduced by IDOMAIN: the user cell of each node (DisType%nodeuser,
    ! 1-based with index_base = 1); the settings carry the grid's shape
    integer(c_int) function gbims_set_dis_nodes(h, nodeuser) &
      bind(C, name='gbims_set_dis_nodes')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), intent(in) :: nodeuser(*)
    end function gbims_set_dis_nodes
    ! ims_base_calc_order (ImsLinearBase.f90:556-610): LORDER/IORDER of RCM
    ! (iord 1) or MD (iord 2), 1-based with index_base = 1; host only (the
    ! handle computes its own ordering at gbims_create)
    integer(c_int) function gbims_calc_order(iord, neq, nja, ia, ja, &
                                             index_base, lorder, iorder) &
      bind(C, name='gbims_calc_order')
      import :: c_int
      integer(c_int), value :: iord, neq, nja, index_base
      integer(c_int), intent(in) :: ia(*), ja(*)
      integer(c_int), intent(out) :: lorder(*), iorder(*)
    end function gbims_calc_order
  end interface

  public :: gbims_calc_order

  !> The GB300 accelerator of one solution
  type :: ImsGb300Type
    type(c_ptr) :: h = c_null_ptr
    integer(I4B) :: neq = 0
    integer(I4B) :: ilinmeth = 1
    integer(I4B) :: nconv = 0
  contains
    procedure :: gb_allocate
    procedure :: gb_apply
    procedure :: gb_deallocate
  end type ImsGb300Type

contains

  !> @brief The library's message for the last error on the handle
  function gb_message(h) result(msg)
    type(c_ptr), intent(in) :: h
    character(len=512) :: msg
    character(kind=c_char), pointer :: s(:)
    type(c_ptr) :: p
    integer(I4B) :: i
    msg = ' '
    p = gbims_last_error(h)
    if (.not. c_associated(p)) return
    call c_f_pointer(p, s, [512])
    do i = 1, 512
      if (s(i) == c_null_char) exit
      msg(i:i) = s(i)
    end do
  end function gb_message

  !> @brief imslinear_allocate: the settings IMS already holds and the
  !! solution's 1-based IA/JA (diagonal first in each row).  The DIS shape is
  !! found from the pattern (nlay = nrow = ncol = 0) unless the solution's one
  !! model is a DIS grid that passes its shape (DIS_SHAPE = nlay, nrow, ncol)
  !! and, with IDOMAIN cells removed, its NODEUSER map; NCONV > 1 asks for the
  !! per-inner-iteration records of CONVNMOD models starting at CONVMODSTART.
  subroutine gb_allocate(this, dvclose, rclose, icnvgopt, iter1, ilinmeth, &
                         iscl, iord, north, relax, level, droptol, neq, nja, &
                         ia, ja, nconv, convnmod, convmodstart, dis_shape, &
                         nodeuser)
    class(ImsGb300Type), intent(inout) :: this
    real(DP), intent(in) :: dvclose, rclose, relax, droptol
    integer(I4B), intent(in) :: icnvgopt, iter1, ilinmeth, iscl, iord, north
    integer(I4B), intent(in) :: level, neq, nja, nconv, convnmod
    integer(I4B), dimension(neq + 1), intent(in) :: ia
    integer(I4B), dimension(nja), intent(in) :: ja
    integer(I4B), dimension(convnmod + 1), intent(in) :: convmodstart
    integer(I4B), dimension(3), intent(in), optional :: dis_shape
    integer(I4B), dimension(:), intent(in), optional :: nodeuser
    type(gbims_settings_t) :: s
    integer(c_int) :: ierr
    s%dvclose = dvclose
    s%rclose = rclose
    s%icnvgopt = icnvgopt
    s%iter1 = iter1
    s%ilinmeth = ilinmeth
    s%iscl = iscl
    s%iord = iord
    s%north = north
    s%relax = relax
    s%level = level
    s%droptol = droptol
    s%precision = GBIMS_FP64
    s%index_base = 1
    s%nlay = 0
    s%nrow = 0
    s%ncol = 0
    if (present(dis_shape)) then
      s%nlay = dis_shape(1)
      s%nrow = dis_shape(2)
      s%ncol = dis_shape(3)
    end if
    ierr = gbims_create(s, neq, nja, ia, ja, this%h)
    if (ierr < 0) then
      call store_error('GB300 IMS allocation failed: '// &
                       trim(gb_message(this%h)), terminate=.TRUE.)
    end if
    if (present(dis_shape) .and. present(nodeuser)) then
      if (neq < dis_shape(1) * dis_shape(2) * dis_shape(3)) then
        ierr = gbims_set_dis_nodes(this%h, nodeuser)
        if (ierr < 0) then
          call store_error('GB300 IMS node map: '//trim(gb_message(this%h)), &
                           terminate=.TRUE.)
        end if
      end if
    end if
    this%neq = neq
    this%ilinmeth = ilinmeth
    this%nconv = nconv
    if (nconv > 1) then
      ierr = gbims_set_inner_records(this%h, nconv, convnmod, convmodstart)
      if (ierr < 0) then
        call store_error('GB300 IMS records: '//trim(gb_message(this%h)), &
                         terminate=.TRUE.)
      end if
    end if
  end subroutine gb_allocate

  !> @brief imslinear_ap: one linear solve of the solution's system
  subroutine gb_apply(this, icnvg, kstp, kiter, in_iter, nconv, convnmod, &
                      caccel, summary, amat, rhs, x, iout)
    class(ImsGb300Type), intent(inout) :: this
    integer(I4B), intent(inout) :: icnvg
    integer(I4B), intent(in) :: kstp, kiter, nconv, convnmod, iout
    integer(I4B), intent(inout) :: in_iter
    character(len=31), dimension(nconv), intent(inout) :: caccel
    type(ConvergenceSummaryType), pointer, intent(in) :: summary
    real(DP), dimension(:), intent(inout) :: amat, rhs, x
    type(gbims_summary_t) :: summ
    integer(c_int) :: ierr, cnv, nit, nrec, cap
    integer(I4B) :: k, im, n
    integer(c_int), allocatable :: itin(:), ldv(:), lr(:)
    real(c_double), allocatable :: al(:), om(:), dv(:), rm(:)
    character(len=15) :: cval1, cval2
    ! the record index runs over the outer iterations of a time step
    ! (ImsLinear.f90:676-679)
    if (kiter == 1) summary%iter_cnt = 0
    ierr = gbims_apply(this%h, amat, rhs, x, kstp, kiter, cnv, nit, summ)
    if (ierr < 0) then
      call store_error('GB300 IMS apply failed: '//trim(gb_message(this%h)), &
                       terminate=.TRUE.)
    end if
    if (ierr == GBIMS_WARN_PIVOT .and. iout > 0) then
      write (iout, '(1x,a,i0,a)') 'GB300 IMS: ', summ%pivot_retries, &
        ' ILU pivot retries (delta increased)'
    end if
    icnvg = cnv
    in_iter = nit
    if (nconv > 1 .and. nit > 0) then
      cap = min(nit, nconv - summary%iter_cnt)
      if (cap > 0) then
        allocate (itin(cap), al(cap), om(cap))
        allocate (ldv(cap * convnmod), dv(cap * convnmod))
        allocate (lr(cap * convnmod), rm(cap * convnmod))
        ierr = gbims_get_inner_records(this%h, cap, nrec, itin, al, om, ldv, &
                                       dv, lr, rm)
        if (ierr < 0) then
          call store_error('GB300 IMS records: '//trim(gb_message(this%h)), &
                           terminate=.TRUE.)
        end if
        do k = 1, nrec
          n = summary%iter_cnt + k
          summary%itinner(n) = itin(k)
          write (cval1, '(g15.7)') al(k)
          if (this%ilinmeth == 2) then
            write (cval2, '(g15.7)') om(k)
            caccel(n) = trim(adjustl(cval1))//','//trim(adjustl(cval2))
          else
            caccel(n) = cval1
          end if
          do im = 1, convnmod
            summary%convdvmax(im, n) = dv((k - 1) * convnmod + im)
            summary%convlocdv(im, n) = ldv((k - 1) * convnmod + im)
            summary%convrmax(im, n) = rm((k - 1) * convnmod + im)
            summary%convlocr(im, n) = lr((k - 1) * convnmod + im)
          end do
        end do
        if (nrec > 0) then
          do im = 1, convnmod
            summary%dvmax(im) = dv((nrec - 1) * convnmod + im)
            summary%locdv(im) = ldv((nrec - 1) * convnmod + im)
            summary%rmax(im) = rm((nrec - 1) * convnmod + im)
            summary%locr(im) = lr((nrec - 1) * convnmod + im)
          end do
        end if
        deallocate (itin, al, om, ldv, dv, lr, rm)
      end if
    end if
    summary%iter_cnt = summary%iter_cnt + nit
  end subroutine gb_apply

  !> @brief imslinear_da
  subroutine gb_deallocate(this)
    class(ImsGb300Type), intent(inout) :: this
    integer(c_int) :: ierr
    if (c_associated(this%h)) ierr = gbims_destroy(this%h)
    this%h = c_null_ptr
  end subroutine gb_deallocate

end module ImsGb300Module
