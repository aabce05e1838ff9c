!==============================================================================!
!   Drop-in replacement for the T-FlowS solver files Process/CG.f90,          !
!   BiCG.f90, CGS.f90, Prec1.f90 and Resid.f90: the same subroutine names     !
!   and dummy arguments, forwarding to libtflows_krylov.so (GB300 CUDA        !
!   solver) through ISO_C_BINDING.  Compile with the code's usual flags       !
!   (-fdefault-real-8: REAL is C_DOUBLE, INTEGER is C_INT) in place of the    !
!   five files and link -ltflows_krylov.  The call sites (CalcPS.f90:217,     !
!   CalcZmix.f90:394, NewUVW.f90:506) and their interface blocks stay as      !
!   they are.                                                                 !
!==============================================================================!
MODULE tflows_krylov_c
  USE ISO_C_BINDING, ONLY: C_INT, C_DOUBLE
  IMPLICIT NONE
  INTERFACE
    SUBROUTINE tflows_cg(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,        &
                         prec, niter, tol, IniRes, FinRes) BIND(C, NAME="tflows_cg")
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT) :: N, NB, NONZ, prec, niter
      INTEGER(C_INT) :: Acol(*), Arow(*), Adia(*)
      REAL(C_DOUBLE) :: A(*), Ab(*), x(*), r1(*), tol, IniRes, FinRes
    END SUBROUTINE tflows_cg
    SUBROUTINE tflows_bicg(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,      &
                           prec, niter, tol, IniRes, FinRes) BIND(C, NAME="tflows_bicg")
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT) :: N, NB, NONZ, prec, niter
      INTEGER(C_INT) :: Acol(*), Arow(*), Adia(*)
      REAL(C_DOUBLE) :: A(*), Ab(*), x(*), r1(*), tol, IniRes, FinRes
    END SUBROUTINE tflows_bicg
    SUBROUTINE tflows_cgs(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,       &
                          prec, niter, tol, IniRes, FinRes) BIND(C, NAME="tflows_cgs")
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT) :: N, NB, NONZ, prec, niter
      INTEGER(C_INT) :: Acol(*), Arow(*), Adia(*)
      REAL(C_DOUBLE) :: A(*), Ab(*), x(*), r1(*), tol, IniRes, FinRes
    END SUBROUTINE tflows_cgs
    SUBROUTINE tflows_prec1(N, NONZ, A, Acol, Arow, Adia, D, prec)           &
                           BIND(C, NAME="tflows_prec1")
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT) :: N, NONZ, prec
      INTEGER(C_INT) :: Acol(*), Arow(*), Adia(*)
      REAL(C_DOUBLE) :: A(*), D(*)
    END SUBROUTINE tflows_prec1
    SUBROUTINE tflows_resid(N, NB, NONZ, A, Acol, Arow, Ab, x, r1)           &
                           BIND(C, NAME="tflows_resid")
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT) :: N, NB, NONZ
      INTEGER(C_INT) :: Acol(*), Arow(*)
      REAL(C_DOUBLE) :: A(*), Ab(*), x(*), r1(*)
    END SUBROUTINE tflows_resid
    INTEGER(C_INT) FUNCTION tflows_last_status() BIND(C, NAME="tflows_last_status")
      IMPORT :: C_INT
    END FUNCTION tflows_last_status
  END INTERFACE
END MODULE tflows_krylov_c

!------------------------------------------------------------------------------!
SUBROUTINE cg(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,                     &
              prec, niter, tol, IniRes, FinRes)
  USE tflows_krylov_c, ONLY: tflows_cg
  IMPLICIT NONE
  INTEGER :: N, NB, NONZ
  REAL    :: A(NONZ), Ab(-NB:-1)
  INTEGER :: Acol(N+1), Adia(N), Arow(NONZ)
  REAL    :: x(-NB:N), r1(N)
  INTEGER :: prec, niter
  REAL    :: tol, IniRes, FinRes
  CALL tflows_cg(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,                  &
                 prec, niter, tol, IniRes, FinRes)
END SUBROUTINE cg

SUBROUTINE bicg(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,                   &
                prec, niter, tol, IniRes, FinRes)
  USE tflows_krylov_c, ONLY: tflows_bicg
  IMPLICIT NONE
  INTEGER :: N, NB, NONZ
  REAL    :: A(NONZ), Ab(-NB:-1)
  INTEGER :: Acol(N+1), Adia(N), Arow(NONZ)
  REAL    :: x(-NB:N), r1(N)
  INTEGER :: prec, niter
  REAL    :: tol, IniRes, FinRes
  CALL tflows_bicg(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,                &
                   prec, niter, tol, IniRes, FinRes)
END SUBROUTINE bicg

SUBROUTINE CGS(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,                    &
               prec, Niter, tol, IniRes, FinRes)
  USE tflows_krylov_c, ONLY: tflows_cgs
  IMPLICIT NONE
  INTEGER :: N, NB, NONZ
  REAL    :: A(NONZ), Ab(-NB:-1)
  INTEGER :: Acol(N+1), Adia(N), Arow(NONZ)
  REAL    :: x(-NB:N), r1(N)
  INTEGER :: prec, Niter
  REAL    :: tol, IniRes, FinRes
  CALL tflows_cgs(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1,                 &
                  prec, Niter, tol, IniRes, FinRes)
END SUBROUTINE CGS

SUBROUTINE Prec1(N, NONZ, A, Acol, Arow, Adia, D, prec)
  USE tflows_krylov_c, ONLY: tflows_prec1
  IMPLICIT NONE
  INTEGER :: N, NONZ, prec
  REAL    :: A(NONZ), D(N)
  INTEGER :: Acol(N+1), Adia(N), Arow(NONZ)
  CALL tflows_prec1(N, NONZ, A, Acol, Arow, Adia, D, prec)
END SUBROUTINE Prec1

SUBROUTINE Resid(N, NB, NONZ, A, Acol, Arow, Ab, x, r1)
  USE tflows_krylov_c, ONLY: tflows_resid
  IMPLICIT NONE
  INTEGER :: N, NB, NONZ
  REAL    :: A(NONZ), Ab(-NB:-1)
  INTEGER :: Acol(N+1), Arow(NONZ)
  REAL    :: x(-NB:N), r1(N)
  CALL tflows_resid(N, NB, NONZ, A, Acol, Arow, Ab, x, r1)
END SUBROUTINE Resid
