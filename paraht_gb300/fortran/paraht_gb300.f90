! paraht_gb300.f90 -- Fortran drop-in for the reduction path, calling libparaht (include/paraht.h)
! through ISO_C_BINDING.
!
! The modules `ab2rht` and `rht2ht` export `ab2rht_simple`, `rht2ht_householder` and
! `rht2ht_givens` with exactly the argument lists of the reference (src/ab2rht.f90:8-13,
! src/rht2ht.f90:1346-1351, src/rht2ht.f90:696-700), so a
! caller such as src/profilereduction.f90 only needs to be recompiled against this file and
! linked with -lparaht.  Module `paraht_qz` adds `hgeqz_eigs`, the eigenvalues of the reduced
! pencil (no counterpart in the reference).  Arrays stay on the host; each call copies them to the GPU, reduces and
! copies them back.  An optional trailing INFO argument returns the library status (0 = ok,
! -i = i-th argument invalid, <= -1000 = PARAHT_ERR_*); without it a failure is reported on
! standard error (the reference itself performs no error reporting).
!
! Build (not done by this repository: the image has no Fortran compiler):
!   gfortran -O2 -c paraht_gb300.f90
!   gfortran ... your_program.f90 paraht_gb300.o -L<dir of libparaht.so> -lparaht -Wl,-rpath,<dir>

module paraht_c
   use iso_c_binding, only: c_int, c_double, c_char, c_ptr
   implicit none
   interface
      integer(c_int) function paraht_ab2rht(n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, time_components) &
         bind(C, name="paraht_ab2rht")
         import :: c_int, c_double
         integer(c_int), value :: n, lda, ldb, ldq, ldz, nb, p, time_components
         real(c_double) :: A(*), B(*), Q(*), Z(*)
      end function paraht_ab2rht

      integer(c_int) function paraht_rht2ht(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, time_components) &
         bind(C, name="paraht_rht2ht")
         import :: c_int, c_double
         integer(c_int), value :: n, lda, ldb, ldq, ldz, r, nq, time_components
         real(c_double) :: A(*), B(*), Q(*), Z(*)
      end function paraht_rht2ht

      integer(c_int) function paraht_rht2ht_givens(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq) &
         bind(C, name="paraht_rht2ht_givens")
         import :: c_int, c_double
         integer(c_int), value :: n, lda, ldb, ldq, ldz, r, nq
         real(c_double) :: A(*), B(*), Q(*), Z(*)
      end function paraht_rht2ht_givens

      integer(c_int) function paraht_reduce(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags) &
         bind(C, name="paraht_reduce")
         import :: c_int, c_double
         integer(c_int), value :: n, lda, ldb, ldq, ldz, r, p, nq, flags
         real(c_double) :: A(*), B(*), Q(*), Z(*)
      end function paraht_reduce

      ! LAPACK DGGHD3's arguments (without the work array) plus r, p, nq, flags
      integer(c_int) function paraht_gghd3(compq, compz, n, ilo, ihi, A, lda, B, ldb, Q, ldq, Z, ldz, &
                                           r, p, nq, flags) bind(C, name="paraht_gghd3")
         import :: c_int, c_double, c_char
         character(kind=c_char), value :: compq, compz
         integer(c_int), value :: n, ilo, ihi, lda, ldb, ldq, ldz, r, p, nq, flags
         real(c_double) :: A(*), B(*), Q(*), Z(*)
      end function paraht_gghd3

      ! QZ eigenvalues of count Hessenberg-triangular pencils (arrays of per-pencil pointers)
      integer(c_int) function paraht_hgeqz_eigs(count, n, H, ldh, T, ldt, alphar, alphai, beta, info) &
         bind(C, name="paraht_hgeqz_eigs")
         import :: c_int, c_ptr
         integer(c_int), value :: count
         integer(c_int) :: n(*), ldh(*), ldt(*), info(*)
         type(c_ptr) :: H(*), T(*), alphar(*), alphai(*), beta(*)
      end function paraht_hgeqz_eigs
   end interface

contains

   subroutine paraht_report(who, status, info)
      character(len=*), intent(in) :: who
      integer(c_int), intent(in) :: status
      integer, intent(out), optional :: info
      if (present(info)) then
         info = int(status)
      else if (status /= 0) then
         write(0, '(A,A,I0)') who, ': libparaht status ', status
      end if
   end subroutine paraht_report

end module paraht_c

module ab2rht
   use paraht_c
   implicit none
contains
   ! src/ab2rht.f90:8 -- stage 1, (A, B) -> (r-Hessenberg, upper triangular); Q <- Q*Q1, Z <- Z*Z1
   subroutine ab2rht_simple(n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, time_components, info)
      integer, intent(in) :: n, lda, ldb, ldq, ldz, nb, p
      double precision, intent(inout) :: A(lda,*), B(ldb,*), Z(ldz,*), Q(ldq,*)
      logical :: time_components
      integer, intent(out), optional :: info
      integer(c_int) :: status, tc
      tc = 0
      if (time_components) tc = 1
      status = paraht_ab2rht(int(n, c_int), A, int(lda, c_int), B, int(ldb, c_int), Q, int(ldq, c_int), &
         Z, int(ldz, c_int), int(nb, c_int), int(p, c_int), tc)
      call paraht_report('ab2rht_simple', status, info)
   end subroutine ab2rht_simple
end module ab2rht

module rht2ht
   use paraht_c
   implicit none
contains
   ! src/rht2ht.f90:1346 -- stage 2, r-Hessenberg -> Hessenberg; Q, Z accumulated
   subroutine rht2ht_householder(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, time_components, info)
      integer, intent(in) :: n, lda, ldb, ldq, ldz, r, nq
      double precision, intent(inout) :: A(lda,*), B(ldb,*), Z(ldz,*), Q(ldq,*)
      logical :: time_components
      integer, intent(out), optional :: info
      integer(c_int) :: status, tc
      tc = 0
      if (time_components) tc = 1
      status = paraht_rht2ht(int(n, c_int), A, int(lda, c_int), B, int(ldb, c_int), Q, int(ldq, c_int), &
         Z, int(ldz, c_int), int(r, c_int), int(nq, c_int), tc)
      call paraht_report('rht2ht_householder', status, info)
   end subroutine rht2ht_householder

   ! src/rht2ht.f90:696 -- stage 2 with Givens rotations (r <= 32, r + nq <= 64 on the GPU)
   subroutine rht2ht_givens(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, info)
      integer, intent(in) :: n, lda, ldb, ldq, ldz, r, nq
      double precision, intent(inout) :: A(lda,*), B(ldb,*), Z(ldz,*), Q(ldq,*)
      integer, intent(out), optional :: info
      integer(c_int) :: status
      status = paraht_rht2ht_givens(int(n, c_int), A, int(lda, c_int), B, int(ldb, c_int), Q, int(ldq, c_int), &
         Z, int(ldz, c_int), int(r, c_int), int(nq, c_int))
      call paraht_report('rht2ht_givens', status, info)
   end subroutine rht2ht_givens
end module rht2ht

module paraht_qz
   use paraht_c
   use iso_c_binding, only: c_int, c_ptr, c_loc
   implicit none
contains
   ! Eigenvalues of one Hessenberg-triangular pencil (H, T) on the GPU, the step after the
   ! reduction (LAPACK DHGEQZ with JOB='E', COMPQ=COMPZ='N'; no counterpart in the reference):
   ! eigenvalue j is (alphar(j) + i alphai(j)) / beta(j), beta(j) >= 0, beta(j) = 0 for an
   ! infinite one.  H and T are not modified.  info: 0, 2 (no convergence), else a library status.
   subroutine hgeqz_eigs(n, H, ldh, T, ldt, alphar, alphai, beta, info)
      integer, intent(in) :: n, ldh, ldt
      double precision, intent(in), target :: H(ldh,*), T(ldt,*)
      double precision, intent(out), target :: alphar(*), alphai(*), beta(*)
      integer, intent(out), optional :: info
      integer(c_int) :: status, cn(1), cldh(1), cldt(1), cinfo(1)
      type(c_ptr) :: pH(1), pT(1), pr(1), pi(1), pb(1)
      if (n < 0) then
         status = -3
      else if (n == 0) then
         status = 0
      else
         cn(1) = int(n, c_int)
         cldh(1) = int(ldh, c_int)
         cldt(1) = int(ldt, c_int)
         pH(1) = c_loc(H(1,1))
         pT(1) = c_loc(T(1,1))
         pr(1) = c_loc(alphar(1))
         pi(1) = c_loc(alphai(1))
         pb(1) = c_loc(beta(1))
         status = paraht_hgeqz_eigs(1_c_int, cn, pH, cldh, pT, cldt, pr, pi, pb, cinfo)
         if (status == 0) status = cinfo(1)
      end if
      call paraht_report('hgeqz_eigs', status, info)
   end subroutine hgeqz_eigs
end module paraht_qz
