!> @file
!> iso_c_binding interfaces of the GB300 RI-MP2 library (librimp2_gpu_gb300.so).
!> Same style as the reference's gpu_interfaces.F90 (bind(C,name=...), C_PTR /
!> C_INT / C_DOUBLE); each subroutine of RIMP2.F90 has a drop-in with the same
!> argument list.  Integers and arrays are passed by reference, exactly as the
!> Fortran CONTAINS subroutines receive them, so a call
!>     call RIMP2_calc_toccA(nvirt,nocc,noccEOS,NBA,Calpha,EVocc,EVvirt,tocc,UoccEOST)
!> becomes
!>     stat = rimp2_calc_tocca(nvirt,nocc,noccEOS,NBA,Calpha,EVocc,EVvirt,tocc,UoccEOST)
!> Every function returns an integer status (0 = success); see rimp2_gpu.h.
module rimp2_gpu_interfaces

  use iso_c_binding
  implicit none

  integer(C_INT), parameter :: RIMP2_OK = 0
  integer(C_INT), parameter :: RIMP2_PREC_FP64 = 0
  integer(C_INT), parameter :: RIMP2_PREC_SPLIT = 1

  interface

     ! RIMP2_calc_toccA (RIMP2.F90:381-417)
     integer(C_INT) function rimp2_calc_tocca(nvirt, nocc, noccEOS, NBA, Calpha, EVocc, EVvirt, &
          & tocc, UoccEOST) bind(C, name="rimp2_calc_tocca")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, nocc, noccEOS, NBA
       real(C_DOUBLE), intent(in) :: Calpha(NBA,nvirt,nocc), EVocc(nocc), EVvirt(nvirt)
       real(C_DOUBLE), intent(inout) :: tocc(nocc,noccEOS,nvirt,nvirt)
       real(C_DOUBLE), intent(in) :: UoccEOST(nocc,noccEOS)
     end function rimp2_calc_tocca

     ! RIMP2_calc_tvirtA (RIMP2.F90:419-453)
     integer(C_INT) function rimp2_calc_tvirta(nvirt, nocc, nvirtEOS, NBA, Calpha, EVocc, EVvirt, &
          & tvirt, UvirtEOST) bind(C, name="rimp2_calc_tvirta")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, nocc, nvirtEOS, NBA
       real(C_DOUBLE), intent(in) :: Calpha(NBA,nvirt,nocc), EVocc(nocc), EVvirt(nvirt)
       real(C_DOUBLE), intent(inout) :: tvirt(nocc,nocc,nvirtEOS,nvirt)
       real(C_DOUBLE), intent(in) :: UvirtEOST(nvirt,nvirtEOS)
     end function rimp2_calc_tvirta

     ! RIMP2_calc_toccB (RIMP2.F90:456-481)
     integer(C_INT) function rimp2_calc_toccb(nvirt, noccEOS, tocc, UvirtT, toccEOS) &
          & bind(C, name="rimp2_calc_toccb")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, noccEOS
       real(C_DOUBLE), intent(in) :: tocc(noccEOS,noccEOS,nvirt,nvirt), UvirtT(nvirt,nvirt)
       real(C_DOUBLE), intent(inout) :: toccEOS(nvirt,noccEOS,nvirt,noccEOS)
     end function rimp2_calc_toccb

     ! RIMP2_calc_tvirtB (RIMP2.F90:483-508)
     integer(C_INT) function rimp2_calc_tvirtb(nvirtEOS, nocc, tvirt, UoccT, tvirtEOS) &
          & bind(C, name="rimp2_calc_tvirtb")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirtEOS, nocc
       real(C_DOUBLE), intent(in) :: tvirt(nocc,nocc,nvirtEOS,nvirtEOS), UoccT(nocc,nocc)
       real(C_DOUBLE), intent(inout) :: tvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc)
     end function rimp2_calc_tvirtb

     ! RIMP2_TransAlpha1 (RIMP2.F90:510-533)
     integer(C_INT) function rimp2_transalpha1(nvirt, noccEOS, nba, UvirtT, AlphaCD4, AlphaCD5) &
          & bind(C, name="rimp2_transalpha1")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, noccEOS, nba
       real(C_DOUBLE), intent(in) :: UvirtT(nvirt,nvirt), AlphaCD4(nba,nvirt,noccEOS)
       real(C_DOUBLE), intent(inout) :: AlphaCD5(nba,nvirt,noccEOS)
     end function rimp2_transalpha1

     ! RIMP2_TransAlpha2 (RIMP2.F90:536-560)
     integer(C_INT) function rimp2_transalpha2(n2, n1, n3, nba, U, AlphaCD4, AlphaCD5) &
          & bind(C, name="rimp2_transalpha2")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: n2, n1, n3, nba
       real(C_DOUBLE), intent(in) :: U(n1,n3), AlphaCD4(nba,n1,n2)
       real(C_DOUBLE), intent(inout) :: AlphaCD5(nba,n3,n2)
     end function rimp2_transalpha2

     ! RIMP2_calc_gocc (RIMP2.F90:562-587)
     integer(C_INT) function rimp2_calc_gocc(nvirt, noccEOS, NBA, Calpha3, goccEOS) &
          & bind(C, name="rimp2_calc_gocc")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, noccEOS, NBA
       real(C_DOUBLE), intent(in) :: Calpha3(NBA,nvirt,noccEOS)
       real(C_DOUBLE), intent(inout) :: goccEOS(nvirt,noccEOS,nvirt,noccEOS)
     end function rimp2_calc_gocc

     ! RIMP2_calc_gvirt (RIMP2.F90:589-614)
     integer(C_INT) function rimp2_calc_gvirt(nvirtEOS, nocc, NBA, Calpha3, gvirtEOS) &
          & bind(C, name="rimp2_calc_gvirt")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirtEOS, nocc, NBA
       real(C_DOUBLE), intent(in) :: Calpha3(NBA,nvirtEOS,nocc)
       real(C_DOUBLE), intent(inout) :: gvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc)
     end function rimp2_calc_gvirt

     ! RIMP2_calc_gen4DimFO (RIMP2.F90:616-641)
     integer(C_INT) function rimp2_calc_gen4dimfo(NBA, Calpha3, n1, n2, Calpha4, n3, n4, djik) &
          & bind(C, name="rimp2_calc_gen4dimfo")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: NBA, n1, n2, n3, n4
       real(C_DOUBLE), intent(in) :: Calpha3(NBA,n1,n2), Calpha4(NBA,n3,n4)
       real(C_DOUBLE), intent(inout) :: djik(n1,n2,n3,n4)
     end function rimp2_calc_gen4dimfo

     ! the driver's dgemm calls (RIMP2.F90:79,87,110,118,137,160)
     integer(C_INT) function rimp2_dgemm(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, &
          & C, ldc) bind(C, name="rimp2_dgemm")
       import :: C_INT, C_DOUBLE, C_CHAR
       character(kind=C_CHAR), intent(in) :: transa, transb
       integer(C_INT), intent(in) :: m, n, k, lda, ldb, ldc
       real(C_DOUBLE), intent(in) :: alpha, beta
       real(C_DOUBLE), intent(in) :: A(lda,*), B(ldb,*)
       real(C_DOUBLE), intent(inout) :: C(ldc,*)
     end function rimp2_dgemm

     ! Steps 5-8 of the driver in one call (RIMP2.F90:71-170)
     integer(C_INT) function rimp2_steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, Calpha, EVocc, &
          & EVvirt, UoccEOST, UvirtT, UoccT, UvirtEOST, toccEOS, tvirtEOS, goccEOS, gvirtEOS) &
          & bind(C, name="rimp2_steps5to8")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, nocc, noccEOS, nvirtEOS, NBA
       real(C_DOUBLE), intent(in) :: Calpha(NBA,nvirt,nocc), EVocc(nocc), EVvirt(nvirt)
       real(C_DOUBLE), intent(in) :: UoccEOST(nocc,noccEOS), UvirtT(nvirt,nvirt)
       real(C_DOUBLE), intent(in) :: UoccT(nocc,nocc), UvirtEOST(nvirt,nvirtEOS)
       real(C_DOUBLE), intent(inout) :: toccEOS(nvirt,noccEOS,nvirt,noccEOS)
       real(C_DOUBLE), intent(inout) :: tvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc)
       real(C_DOUBLE), intent(inout) :: goccEOS(nvirt,noccEOS,nvirt,noccEOS)
       real(C_DOUBLE), intent(inout) :: gvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc)
     end function rimp2_steps5to8

     ! fused fragment energies (occupied and virtual partitioning) for general U
     integer(C_INT) function rimp2_energy_eos(nvirt, nocc, noccEOS, nvirtEOS, NBA, Calpha, EVocc, &
          & EVvirt, UoccEOST, UvirtT, UoccT, UvirtEOST, Eocc, Evirt, precision) &
          & bind(C, name="rimp2_energy_eos")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, nocc, noccEOS, nvirtEOS, NBA, precision
       real(C_DOUBLE), intent(in) :: Calpha(NBA,nvirt,nocc), EVocc(nocc), EVvirt(nvirt)
       real(C_DOUBLE), intent(in) :: UoccEOST(nocc,noccEOS), UvirtT(nvirt,nvirt)
       real(C_DOUBLE), intent(in) :: UoccT(nocc,nocc), UvirtEOST(nvirt,nvirtEOS)
       real(C_DOUBLE), intent(out) :: Eocc, Evirt
     end function rimp2_energy_eos

     ! first-order block of the driver (RIMP2.F90:172-251); pass UoccT as UoccallT
     integer(C_INT) function rimp2_first_order(nvirt, nocc, noccEOS, nvirtEOS, nocctot, NBA, &
          & Calpha, CalphaOcc, CalphaVV, UoccEOST, UvirtT, UoccT, UoccallT, UvirtEOST, djik, blad) &
          & bind(C, name="rimp2_first_order")
       import :: C_INT, C_DOUBLE
       integer(C_INT), intent(in) :: nvirt, nocc, noccEOS, nvirtEOS, nocctot, NBA
       real(C_DOUBLE), intent(in) :: Calpha(NBA,nvirt,nocc), CalphaOcc(NBA,nocc,nocctot)
       real(C_DOUBLE), intent(in) :: CalphaVV(NBA,nvirt,nvirt), UoccEOST(nocc,noccEOS)
       real(C_DOUBLE), intent(in) :: UvirtT(nvirt,nvirt), UoccT(nocc,nocc)
       real(C_DOUBLE), intent(in) :: UoccallT(nocctot,nocctot), UvirtEOST(nvirt,nvirtEOS)
       real(C_DOUBLE), intent(inout) :: djik(nvirt,noccEOS,noccEOS,nocctot)
       real(C_DOUBLE), intent(inout) :: blad(nvirtEOS,nocc,nvirtEOS,nvirt)
     end function rimp2_first_order

     ! MP2 pair and total energy (FP64 or split precision); tamp may be C_NULL_PTR
     integer(C_INT) function rimp2_energy(nvirt, nocc, NBA, Calpha, EVocc, EVvirt, Epair, Etot, &
          & tamp, precision) bind(C, name="rimp2_energy")
       import :: C_INT, C_DOUBLE, C_PTR
       integer(C_INT), intent(in) :: nvirt, nocc, NBA, precision
       real(C_DOUBLE), intent(in) :: Calpha(NBA,nvirt,nocc), EVocc(nocc), EVvirt(nvirt)
       real(C_DOUBLE), intent(inout) :: Epair(nocc,nocc), Etot
       type(C_PTR), value :: tamp
     end function rimp2_energy

     ! device-pointer form (host_data use_device addresses), stream = acc_get_cuda_stream(q)
     integer(C_INT) function rimp2_energy_dev(nvirt, nocc, NBA, dCalpha, dEVocc, dEVvirt, &
          & dEpair, dEtot, dtamp, precision, stream) bind(C, name="rimp2_energy_dev")
       import :: C_INT, C_PTR
       integer(C_INT), value :: nvirt, nocc, NBA, precision
       type(C_PTR), value :: dCalpha, dEVocc, dEVvirt, dEpair, dEtot, dtamp, stream
     end function rimp2_energy_dev

     ! total / free device memory (replaces get_dev_mem, gpu_interfaces.F90:47-53)
     integer(C_INT) function rimp2_get_dev_mem(total, free) bind(C, name="rimp2_get_dev_mem")
       import :: C_INT, C_SIZE_T
       integer(C_SIZE_T), intent(out) :: total, free
     end function rimp2_get_dev_mem

     ! route work to a caller stream (e.g. acc_get_cuda_stream(async_id(1)))
     integer(C_INT) function rimp2_set_stream(stream) bind(C, name="rimp2_set_stream")
       import :: C_INT, C_PTR
       type(C_PTR), value :: stream
     end function rimp2_set_stream

     ! energy kernel of the last split launch: 0 none, 1 one-CTA, 2 paired-CTA
     integer(C_INT) function rimp2_last_split_kernel() bind(C, name="rimp2_last_split_kernel")
       import :: C_INT
     end function rimp2_last_split_kernel

     ! C string of the last error on this thread
     type(C_PTR) function rimp2_last_error_string() bind(C, name="rimp2_last_error_string")
       import :: C_PTR
     end function rimp2_last_error_string

  end interface

end module rimp2_gpu_interfaces
