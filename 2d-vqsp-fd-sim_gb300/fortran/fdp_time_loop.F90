!=======================================================================
! Drop-in replacement of SUBROUTINE TIME_LOOP (time_loop.F90:3-209) that
! runs the time stepping on a GB300 through the C ABI of include/fdp.h.
!
! Build (where a Fortran compiler exists; none is installed where this
! library is built and tested, so this file has not been compiled): add it
! to the reference's serial build after mod_*.F90 and link libfdp.so, then
! call TIME_LOOP_GB300 instead of TIME_LOOP in main.F90:84.  The
! reference's set-up (READ_OPEN .. PPML) runs unchanged and fills the
! modules this routine reads.
!=======================================================================
MODULE FDP_GB300
  ! Host arrays cross the ABI as assumed-size dummies of the reference's own
  ! kinds, passed by reference: the module arrays (ALLOCATABLE without
  ! TARGET, mod_wavefield.F90:19-20, mod_pml.F90:7,17, mod_auxil.F90:33) are
  ! contiguous, so they are handed over as they are, with no address taken
  ! and no copy.  Only the context handle is a C_PTR.
  USE ISO_C_BINDING
  USE PRECISION, ONLY: PP
  IMPLICIT NONE

  TYPE, BIND(C) :: FDP_GRID_T
    INTEGER(C_INT32_T) :: MX, MZ, TPML, STRESS_IMAGING, LIN_X, LIN_Z, PRECISION, DEVICE
    REAL(C_DOUBLE)     :: H, DT, TAU_EPS
  END TYPE FDP_GRID_T

  INTEGER(C_INT32_T), PARAMETER :: FDP_REC_TLV = 1, FDP_REC_TLQ = 2, FDP_REC_TLP = 4
  INTEGER(C_INT32_T), PARAMETER :: FDP_SNAP_UM = 1, FDP_SNAP_WM = 2, FDP_SNAP_QX = 4, FDP_SNAP_QZ = 8

  INTERFACE
    INTEGER(C_INT) FUNCTION FDP_CREATE(G, CTX) BIND(C, NAME='fdp_create')
      IMPORT :: C_INT, C_PTR, FDP_GRID_T
      TYPE(FDP_GRID_T), INTENT(IN) :: G
      TYPE(C_PTR), INTENT(OUT) :: CTX
    END FUNCTION FDP_CREATE
    INTEGER(C_INT) FUNCTION FDP_SET_MEDIUM(CTX, JM, NX, NZ, JMNUM, TABLE24) BIND(C, NAME='fdp_set_medium')
      IMPORT :: C_INT, C_INT32_T, C_PTR, PP
      TYPE(C_PTR), VALUE :: CTX
      INTEGER(C_INT32_T), DIMENSION(*), INTENT(IN) :: JM
      INTEGER(C_INT32_T), VALUE :: NX, NZ, JMNUM
      REAL(PP), DIMENSION(*), INTENT(IN) :: TABLE24
    END FUNCTION FDP_SET_MEDIUM
    INTEGER(C_INT) FUNCTION FDP_SET_PML_ARRAYS(CTX, ODA_XL, ODB_XL, ODC_XL, ODD_XL, ODA_XH, ODB_XH, ODC_XH, ODD_XH, &
        ODA_ZH, ODB_ZH, ODC_ZH, ODD_ZH, ODA2_XL, ODB2_XL, ODC2_XL, ODD2_XL, ODA2_XH, ODB2_XH, ODC2_XH, ODD2_XH, &
        ODA2_ZH, ODB2_ZH, ODC2_ZH, ODD2_ZH) BIND(C, NAME='fdp_set_pml_arrays')
      IMPORT :: C_INT, C_PTR, PP
      TYPE(C_PTR), VALUE :: CTX
      REAL(PP), DIMENSION(*), INTENT(IN) :: ODA_XL, ODB_XL, ODC_XL, ODD_XL, ODA_XH, ODB_XH, ODC_XH, ODD_XH, &
        ODA_ZH, ODB_ZH, ODC_ZH, ODD_ZH, ODA2_XL, ODB2_XL, ODC2_XL, ODD2_XL, ODA2_XH, ODB2_XH, ODC2_XH, ODD2_XH, &
        ODA2_ZH, ODB2_ZH, ODC2_ZH, ODD2_ZH
    END FUNCTION FDP_SET_PML_ARRAYS
    INTEGER(C_INT) FUNCTION FDP_SET_BOTTOM_NR(CTX, AB16) BIND(C, NAME='fdp_set_bottom_nr')
      IMPORT :: C_INT, C_PTR, PP
      TYPE(C_PTR), VALUE :: CTX
      REAL(PP), DIMENSION(16), INTENT(IN) :: AB16
    END FUNCTION FDP_SET_BOTTOM_NR
    INTEGER(C_INT) FUNCTION FDP_SET_SOURCE(CTX, SOURTF, MT2) BIND(C, NAME='fdp_set_source')
      IMPORT :: C_INT, C_INT32_T, C_PTR, PP
      TYPE(C_PTR), VALUE :: CTX
      REAL(PP), DIMENSION(*), INTENT(IN) :: SOURTF
      INTEGER(C_INT32_T), VALUE :: MT2
    END FUNCTION FDP_SET_SOURCE
    INTEGER(C_INT) FUNCTION FDP_SET_RECEIVERS(CTX, IRECX, LRECX, IRECZ, LRECZ, MR, FLAGS) &
        BIND(C, NAME='fdp_set_receivers')
      IMPORT :: C_INT, C_INT32_T, C_PTR
      TYPE(C_PTR), VALUE :: CTX
      INTEGER(C_INT32_T), DIMENSION(*), INTENT(IN) :: IRECX, LRECX, IRECZ, LRECZ
      INTEGER(C_INT32_T), VALUE :: MR, FLAGS
    END FUNCTION FDP_SET_RECEIVERS
    INTEGER(C_INT) FUNCTION FDP_RUN(CTX, IT_BEGIN, IT_END) BIND(C, NAME='fdp_run')
      IMPORT :: C_INT, C_INT32_T, C_PTR
      TYPE(C_PTR), VALUE :: CTX
      INTEGER(C_INT32_T), VALUE :: IT_BEGIN, IT_END
    END FUNCTION FDP_RUN
    INTEGER(C_INT) FUNCTION FDP_GET_RECEIVERS(CTX, IT_FIRST, N_LEVELS, HOST) BIND(C, NAME='fdp_get_receivers')
      IMPORT :: C_INT, C_INT32_T, C_PTR, PP
      TYPE(C_PTR), VALUE :: CTX
      INTEGER(C_INT32_T), VALUE :: IT_FIRST, N_LEVELS
      REAL(PP), DIMENSION(*), INTENT(OUT) :: HOST
    END FUNCTION FDP_GET_RECEIVERS
    INTEGER(C_INT) FUNCTION FDP_GET_SNAPSHOT(CTX, MASK, HOST) BIND(C, NAME='fdp_get_snapshot')
      IMPORT :: C_INT, C_INT32_T, C_PTR, PP
      TYPE(C_PTR), VALUE :: CTX
      INTEGER(C_INT32_T), VALUE :: MASK
      REAL(PP), DIMENSION(*), INTENT(OUT) :: HOST
    END FUNCTION FDP_GET_SNAPSHOT
    TYPE(C_PTR) FUNCTION FDP_LAST_ERROR(CTX) BIND(C, NAME='fdp_last_error')
      IMPORT :: C_PTR
      TYPE(C_PTR), VALUE :: CTX
    END FUNCTION FDP_LAST_ERROR
    SUBROUTINE FDP_DESTROY(CTX) BIND(C, NAME='fdp_destroy')
      IMPORT :: C_PTR
      TYPE(C_PTR), VALUE :: CTX
    END SUBROUTINE FDP_DESTROY
  END INTERFACE

CONTAINS

  ! Mirrors the reference's error convention: message to unit 11, then STOP.
  SUBROUTINE FDP_CHECK(RC, CTX, WHAT)
    INTEGER(C_INT), INTENT(IN) :: RC
    TYPE(C_PTR), INTENT(IN) :: CTX
    CHARACTER(LEN=*), INTENT(IN) :: WHAT
    CHARACTER(KIND=C_CHAR), POINTER :: MSG(:)
    INTEGER :: N
    IF (RC == 0) RETURN
    CALL C_F_POINTER(FDP_LAST_ERROR(CTX), MSG, [512])
    N = 0
    DO WHILE (N < 512)
      IF (MSG(N+1) == C_NULL_CHAR) EXIT
      N = N + 1
    END DO
    WRITE (11,*) '  GB300 ', WHAT, ' FAILED, CODE=', RC, ': ', MSG(1:N)
    STOP
  END SUBROUTINE FDP_CHECK

  SUBROUTINE TIME_LOOP_GB300
    USE PRECISION   , ONLY: PP
    USE CONTROL_DATA, ONLY: KEY_SNV, KEY_TLV, KEY_TLQ, KEY_TLP, MX, MZ, MT1, MT2, DT, TAU_EPS, IPAS2, TPML, &
                            LIN_X, LIN_Z, STRESS_IMAGING, MR, IRECX, LRECX, IRECZ, LRECZ
    USE GRID_MEDIUM , ONLY: JM, JMNUM, H, MU, SIG_XX_1, SIG_XX_2, SIG_XX_3, SIG_ZZ_1, SIG_ZZ_2, SIG_ZZ_3, &
                            PRES_1, PRES_2, PRES_3, REL1_U, REL1_W, REL2_U, REL2_W, REL3_U, REL3_W, &
                            REL1_QX, REL1_QZ, REL2_QX, REL2_QZ, REL3_QX, REL3_QZ, AUXIL_W, AUXIL_QZ
    USE AUXIL       , ONLY: PMLL, PMLXH, PMLZH, SOURTF_A
    USE WAVEFIELD   , ONLY: UM, WM, QX, QZ
    USE PML         , ONLY: ODA_XL, ODB_XL, ODC_XL, ODD_XL, ODA_XH, ODB_XH, ODC_XH, ODD_XH, &
                            ODA_ZH, ODB_ZH, ODC_ZH, ODD_ZH, ODA2_XL, ODB2_XL, ODC2_XL, ODD2_XL, &
                            ODA2_XH, ODB2_XH, ODC2_XH, ODD2_XH, ODA2_ZH, ODB2_ZH, ODC2_ZH, ODD2_ZH
    USE NONREF_BOUND, ONLY: ABW01, ABW02, ABW10, ABW11, ABW12, ABW20, ABW21, ABW22, &
                            ABH01, ABH02, ABH10, ABH11, ABH12, ABH20, ABH21, ABH22
    USE T_LOOP      , ONLY: ITILE
    USE INTERFACES  , ONLY: STORE_SNAPSHOTS

    INTEGER, PARAMETER :: NCHUNK = 500
    TYPE(FDP_GRID_T) :: G
    TYPE(C_PTR) :: CTX
    REAL(PP), ALLOCATABLE :: TAB(:,:), REC(:,:,:)
    REAL(PP) :: AB(16)
    INTEGER(C_INT32_T), ALLOCATABLE :: JMC(:,:), IRX(:), LRX(:), IRZ(:), LRZ(:)
    INTEGER :: IT0, IT1, N, K, J, FLAGS
    LOGICAL :: EX

    G%MX = MX; G%MZ = MZ; G%TPML = TPML; G%LIN_X = LIN_X; G%LIN_Z = LIN_Z
    G%STRESS_IMAGING = MERGE(1, 0, STRESS_IMAGING)
    G%PRECISION = STORAGE_SIZE(1._PP) / 8
    G%DEVICE = 0
    G%H = H; G%DT = DT; G%TAU_EPS = TAU_EPS
    CALL FDP_CHECK(FDP_CREATE(G, CTX), C_NULL_PTR, 'fdp_create')

    ! medium (read_model.F90, read_model_par.F90): JM as 32-bit integers and
    ! the table in .MO record order
    ALLOCATE (JMC(PMLL:PMLXH, 0:PMLZH), TAB(24, JMNUM))
    JMC = INT(JM, C_INT32_T)
    TAB( 1,:) = MU;       TAB( 2,:) = SIG_XX_1; TAB( 3,:) = SIG_XX_2; TAB( 4,:) = SIG_XX_3
    TAB( 5,:) = SIG_ZZ_1; TAB( 6,:) = SIG_ZZ_2; TAB( 7,:) = SIG_ZZ_3; TAB( 8,:) = PRES_1
    TAB( 9,:) = PRES_2;   TAB(10,:) = PRES_3;   TAB(11,:) = REL1_U;   TAB(12,:) = REL1_W
    TAB(13,:) = REL2_U;   TAB(14,:) = REL2_W;   TAB(15,:) = REL3_U;   TAB(16,:) = REL3_W
    TAB(17,:) = REL1_QX;  TAB(18,:) = REL1_QZ;  TAB(19,:) = REL2_QX;  TAB(20,:) = REL2_QZ
    TAB(21,:) = REL3_QX;  TAB(22,:) = REL3_QZ;  TAB(23,:) = AUXIL_W;  TAB(24,:) = AUXIL_QZ
    CALL FDP_CHECK(FDP_SET_MEDIUM(CTX, JMC, PMLXH-PMLL+1, PMLZH+1, JMNUM, TAB), CTX, 'fdp_set_medium')

    ! PPML profiles (ppml.F90:60-83): the module arrays themselves
    CALL FDP_CHECK(FDP_SET_PML_ARRAYS(CTX, ODA_XL, ODB_XL, ODC_XL, ODD_XL, ODA_XH, ODB_XH, ODC_XH, ODD_XH, &
                   ODA_ZH, ODB_ZH, ODC_ZH, ODD_ZH, ODA2_XL, ODB2_XL, ODC2_XL, ODD2_XL, &
                   ODA2_XH, ODB2_XH, ODC2_XH, ODD2_XH, ODA2_ZH, ODB2_ZH, ODC2_ZH, ODD2_ZH), CTX, 'fdp_set_pml_arrays')

    AB = [ABW01, ABW02, ABW10, ABW11, ABW12, ABW20, ABW21, ABW22, &
          ABH01, ABH02, ABH10, ABH11, ABH12, ABH20, ABH21, ABH22]
    CALL FDP_CHECK(FDP_SET_BOTTOM_NR(CTX, AB), CTX, 'fdp_set_bottom_nr')
    CALL FDP_CHECK(FDP_SET_SOURCE(CTX, SOURTF_A, MT2), CTX, 'fdp_set_source')

    FLAGS = 0
    IF (KEY_TLV) FLAGS = IOR(FLAGS, FDP_REC_TLV)
    IF (KEY_TLQ) FLAGS = IOR(FLAGS, FDP_REC_TLQ)
    IF (KEY_TLP) FLAGS = IOR(FLAGS, FDP_REC_TLP)
    IF (KEY_TLV .OR. KEY_TLP) THEN
      ALLOCATE (IRX(MR), LRX(MR), IRZ(MR), LRZ(MR), REC(10, MR, NCHUNK))
      IRX = IRECX; LRX = LRECX; IRZ = IRECZ; LRZ = LRECZ
      CALL FDP_CHECK(FDP_SET_RECEIVERS(CTX, IRX, LRX, IRZ, LRZ, MR, FLAGS), &
                     CTX, 'fdp_set_receivers')
    END IF

    ! DO ITILE = MT1, MT2 (time_loop.F90:65), NCHUNK levels per call; snapshot
    ! levels (MOD(ITILE,IPAS2)==0) end a chunk so the field can be copied
    IT0 = MT1
    DO WHILE (IT0 <= MT2)
      INQUIRE (FILE = 'STOP', EXIST = EX)          ! time_loop.F90:79-86
      IF (EX) THEN
        OPEN (35, FILE='STOP', STATUS='UNKNOWN'); WRITE (35,*) IT0; CLOSE (35)
        STOP
      END IF
      IT1 = MIN(MT2, IT0 + NCHUNK - 1)
      IF (KEY_SNV) IT1 = MIN(IT1, (IT0 / IPAS2 + 1) * IPAS2)
      CALL FDP_CHECK(FDP_RUN(CTX, IT0, IT1), CTX, 'fdp_run')
      N = IT1 - IT0 + 1
      IF (KEY_TLV .OR. KEY_TLP) THEN
        CALL FDP_CHECK(FDP_GET_RECEIVERS(CTX, IT0, N, REC), CTX, 'fdp_get_receivers')
        DO K = 1, N
          DO J = 1, MR                              ! store_seismograms.F90:140-154
            IF (KEY_TLV) THEN
              OPEN (21, FILE='REC_UW_'//TRIM(STR(J))//'.asc', STATUS='UNKNOWN', POSITION='APPEND')
              WRITE (21, '(5(1X,E13.6))') DT*(IT0+K-1), REC(1:4, J, K)
              CLOSE (21)
              IF (KEY_TLQ) THEN
                OPEN (22, FILE='REC_Q_'//TRIM(STR(J))//'.asc', STATUS='UNKNOWN', POSITION='APPEND')
                WRITE (22, '(5(1X,E13.6))') DT*(IT0+K-1), REC(5:8, J, K)
                CLOSE (22)
              END IF
            END IF
            IF (KEY_TLP) THEN                       ! store_seismograms_pressure.F90:76-83
              OPEN (27, FILE='REC_STRESS_'//TRIM(STR(J))//'.asc', STATUS='UNKNOWN', POSITION='APPEND')
              WRITE (27, '(3(1X,E13.6))') DT*(IT0+K-1), REC(9:10, J, K)
              CLOSE (27)
            END IF
          END DO
        END DO
      END IF
      IF (KEY_SNV .AND. MOD(IT1, IPAS2) == 0) THEN
        ! copy the wavefield into the module arrays and let the reference write it
        CALL FDP_CHECK(FDP_GET_SNAPSHOT(CTX, FDP_SNAP_UM, UM), CTX, 'fdp_get_snapshot')
        CALL FDP_CHECK(FDP_GET_SNAPSHOT(CTX, FDP_SNAP_WM, WM), CTX, 'fdp_get_snapshot')
        IF (KEY_TLQ) THEN
          CALL FDP_CHECK(FDP_GET_SNAPSHOT(CTX, FDP_SNAP_QX, QX), CTX, 'fdp_get_snapshot')
          CALL FDP_CHECK(FDP_GET_SNAPSHOT(CTX, FDP_SNAP_QZ, QZ), CTX, 'fdp_get_snapshot')
        END IF
        ITILE = IT1
        CALL STORE_SNAPSHOTS(IT1)
      END IF
      IT0 = IT1 + 1
    END DO
    CALL FDP_DESTROY(CTX)
  END SUBROUTINE TIME_LOOP_GB300

  FUNCTION STR(K)
    INTEGER, INTENT(IN) :: K
    CHARACTER(LEN=20) :: STR
    WRITE (STR, *) K
    STR = ADJUSTL(STR)
  END FUNCTION STR

END MODULE FDP_GB300
