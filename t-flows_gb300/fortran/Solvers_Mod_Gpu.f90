!==============================================================================!
  module Solvers_Mod
!------------------------------------------------------------------------------!
!   Drop-in replacement of Sources/Process/Solvers_Mod.f90 that runs the       !
!   preconditioned Krylov solves on a GB300 through libtfs_gb300.so.           !
!                                                                              !
!   The subroutines keep the names and argument lists of the reference         !
!   (Cg.f90:2-4, Bicg.f90:2-4, Cgs.f90:2-4), so                                !
!     use Solvers_Mod, only: Bicg, Cg, Cgs                                     !
!   in the callers (e.g. Compute_Pressure_Simple.f90:13) compiles unchanged.   !
!   D stays a public module variable: Main.f90:142 builds its topology.        !
!                                                                              !
!   Build: replace Solvers_Mod.f90 and its Solvers_Mod/*.f90 includes in       !
!   Sources/Process/Makefile.am by this file and link -ltfs_gb300.             !
!------------------------------------------------------------------------------!
  use iso_c_binding
  use Matrix_Mod
!------------------------------------------------------------------------------!
  implicit none
!==============================================================================!

  ! Preconditioning "matrix" (kept for Main.f90:142; formed on the device)
  type(Matrix_Type) :: D

  integer, parameter :: TFS_OK = 0, TFS_ERR_NONFINITE = 4

  interface
    integer(c_int) function tfs_cg(n, nnz, row, col, dia, val, x, r1,      &
                                   prec, niter, tol, ini_res, fin_res)      &
                                   bind(C, name="tfs_cg")
      import :: c_int, c_int32_t, c_double
      integer(c_int32_t), value :: n, nnz, prec
      integer(c_int32_t)        :: row(*), col(*), dia(*), niter
      real(c_double)            :: val(*), x(*), r1(*)
      real(c_double),     value :: tol
      real(c_double)            :: ini_res, fin_res
    end function
    integer(c_int) function tfs_bicg(n, nnz, row, col, dia, val, x, r1,    &
                                     prec, niter, tol, ini_res, fin_res)    &
                                     bind(C, name="tfs_bicg")
      import :: c_int, c_int32_t, c_double
      integer(c_int32_t), value :: n, nnz, prec
      integer(c_int32_t)        :: row(*), col(*), dia(*), niter
      real(c_double)            :: val(*), x(*), r1(*)
      real(c_double),     value :: tol
      real(c_double)            :: ini_res, fin_res
    end function
    integer(c_int) function tfs_cgs(n, nnz, row, col, dia, val, x, r1,     &
                                    prec, niter, tol, ini_res, fin_res)     &
                                    bind(C, name="tfs_cgs")
      import :: c_int, c_int32_t, c_double
      integer(c_int32_t), value :: n, nnz, prec
      integer(c_int32_t)        :: row(*), col(*), dia(*), niter
      real(c_double)            :: val(*), x(*), r1(*)
      real(c_double),     value :: tol
      real(c_double)            :: ini_res, fin_res
    end function
    type(c_ptr) function tfs_last_error() bind(C, name="tfs_last_error")
      import :: c_ptr
    end function
    ! TFS_FP64 = 0, TFS_MIXED = 1 for every later Cg / Bicg / Cgs call
    integer(c_int) function tfs_set_default_precision(mode)                 &
                                   bind(C, name="tfs_set_default_precision")
      import :: c_int
      integer(c_int), value :: mode
    end function
  end interface

  contains

!==============================================================================!
  subroutine Check_Status(status, who)
!------------------------------------------------------------------------------!
!   Stops on a library error, as ReaCom.f90:680-684 stops on bad input.        !
!   A non-finite residual is returned like the reference does (NaN carried).   !
!------------------------------------------------------------------------------!
  integer(c_int)   :: status
  character(len=*) :: who
  if(status /= TFS_OK .and. status /= TFS_ERR_NONFINITE) then
    write(*,*) '# ', who, ': libtfs_gb300 status ', status
    stop
  end if
  end subroutine

!==============================================================================!
  subroutine Cg(A, x, r1, prec, niter, tol, ini_res, fin_res)
!------------------------------------------------------------------------------!
!   Preconditioned CG on the GPU (replaces Solvers_Mod/Cg.f90).                !
!------------------------------------------------------------------------------!
  type(Matrix_Type) :: A
  real              :: x(-A % pnt_grid % n_bnd_cells : A % pnt_grid % n_cells)
  real              :: r1(A % pnt_grid % n_cells)
  integer           :: prec, niter
  real              :: tol, ini_res, fin_res
  integer(c_int)    :: status
  integer           :: n
  n = A % pnt_grid % n_cells
  status = tfs_cg(n, A % row(n+1) - 1, A % row, A % col, A % dia, A % val, &
                  x(1), r1, prec, niter, tol, ini_res, fin_res)
  call Check_Status(status, 'Cg')
  end subroutine

!==============================================================================!
  subroutine Bicg(A, x, r1, prec, niter, tol, ini_res, fin_res)
!------------------------------------------------------------------------------!
!   Preconditioned BiCG on the GPU (replaces Solvers_Mod/Bicg.f90).            !
!------------------------------------------------------------------------------!
  type(Matrix_Type) :: A
  real              :: x(-A % pnt_grid % n_bnd_cells : A % pnt_grid % n_cells)
  real              :: r1(A % pnt_grid % n_cells)
  integer           :: prec, niter
  real              :: tol, ini_res, fin_res
  integer(c_int)    :: status
  integer           :: n
  n = A % pnt_grid % n_cells
  status = tfs_bicg(n, A % row(n+1) - 1, A % row, A % col, A % dia, A % val, &
                    x(1), r1, prec, niter, tol, ini_res, fin_res)
  call Check_Status(status, 'Bicg')
  end subroutine

!==============================================================================!
  subroutine Cgs(A, x, r1, prec, niter, tol, ini_res, fin_res)
!------------------------------------------------------------------------------!
!   Preconditioned CGS on the GPU (replaces Solvers_Mod/Cgs.f90).              !
!------------------------------------------------------------------------------!
  type(Matrix_Type) :: A
  real              :: x(-A % pnt_grid % n_bnd_cells : A % pnt_grid % n_cells)
  real              :: r1(A % pnt_grid % n_cells)
  integer           :: prec, niter
  real              :: tol, ini_res, fin_res
  integer(c_int)    :: status
  integer           :: n
  n = A % pnt_grid % n_cells
  status = tfs_cgs(n, A % row(n+1) - 1, A % row, A % col, A % dia, A % val, &
                   x(1), r1, prec, niter, tol, ini_res, fin_res)
  call Check_Status(status, 'Cgs')
  end subroutine

  end module
