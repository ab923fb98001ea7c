! chem_gpu.F -- drop-in CHEM for CMAQ's CCTM that calls libcmaqchem.so through ISO_C_BINDING.
!
! Keeps the reference's operator signature SUBROUTINE CHEM( CONC, JDATE, JTIME, TSTEP )
! (CCTM/src/gas/ros3/rbdriver.F:20, called from CCTM/src/driver/sciproc.F:298).  Compile it
! in place of the gas/ros3 sources (fixed form, 132-column lines, as CCTM's own .F files)
! and link -lcmaqchem.  The C side of every interface below is declared in cmaqchem.h.
! No Fortran compiler exists in the image this library is built on, so this file is not
! compiled by the library's build; tests/test_capi_exports.py checks that it binds the
! header's names.
      MODULE CMAQCHEM_C
        USE ISO_C_BINDING
        IMPLICIT NONE
        TYPE, BIND(C) :: CMAQCHEM_CFG
          TYPE(C_PTR)    :: MECHANISM
          INTEGER(C_INT) :: SOLVER, SCHEDULE
          REAL(C_DOUBLE) :: RTOL, ATOL
          INTEGER(C_INT) :: NCOLS, NROWS, NLAYS, NSPCSD
          TYPE(C_PTR)    :: CGRID_INDEX
          INTEGER(C_INT) :: DEVICE, MAX_ITER
        END TYPE
        TYPE, BIND(C) :: CMAQCHEM_STATS
          INTEGER(C_LONG_LONG) :: ACCEPTED, REJECTED, FAILED_CELLS, SUNLIT_CELLS, SUNLIT_ATTEMPTS
          REAL(C_DOUBLE)       :: DEVICE_MS
        END TYPE
        INTERFACE
          INTEGER(C_INT) FUNCTION cmaqchem_init( CFG, H ) BIND(C, NAME='cmaqchem_init')
            IMPORT; TYPE(CMAQCHEM_CFG), INTENT(IN) :: CFG; TYPE(C_PTR), INTENT(OUT) :: H
          END FUNCTION
          INTEGER(C_INT) FUNCTION cmaqchem_step( H, CONC, TA, QV, DENS, PRES, SEAICE, OSZ,
     &        RJ, KHET, JDATE, JTIME, TSTEP, ST ) BIND(C, NAME='cmaqchem_step')
            IMPORT
            TYPE(C_PTR), VALUE :: H
            REAL(C_FLOAT)      :: CONC(*)
            REAL(C_FLOAT), INTENT(IN)  :: TA(*), QV(*), DENS(*), PRES(*), SEAICE(*), OSZ(*), RJ(*)
            REAL(C_DOUBLE), INTENT(IN) :: KHET(*)
            INTEGER(C_INT), VALUE      :: JDATE, JTIME
            INTEGER(C_INT), INTENT(IN) :: TSTEP(3)
            TYPE(CMAQCHEM_STATS)       :: ST
          END FUNCTION
          INTEGER(C_INT) FUNCTION cmaqchem_last_error( BUF, LEN ) BIND(C, NAME='cmaqchem_last_error')
            IMPORT; CHARACTER(KIND=C_CHAR) :: BUF(*); INTEGER(C_SIZE_T), VALUE :: LEN
          END FUNCTION
        END INTERFACE
      END MODULE CMAQCHEM_C

      SUBROUTINE CHEM( CONC, JDATE, JTIME, TSTEP )
      USE CMAQCHEM_C
      USE RXNS_DATA, ONLY: CGRID_INDEX, NUMB_MECH_SPC
      USE GRID_CONF                      ! NCOLS, NROWS, NLAYS
      USE CGRID_SPCS, ONLY: NSPCSD
      USE RUNTIME_VARS, ONLY: GLBL_RTOL, GLBL_ATOL, LOGDEV
      USE PHOT_MOD, ONLY: RJ
      USE AEROSOL_CHEMISTRY, ONLY: HETCHEM_RATES, KHETERO
      USE CENTRALIZED_IO_MODULE, ONLY: INTERPOLATE_VAR, OCEAN, SZONE
      USE UTILIO_DEFN
      IMPLICIT NONE
      REAL, POINTER :: CONC( :,:,:,: )
      INTEGER JDATE, JTIME, TSTEP( 3 )
      TYPE(C_PTR), SAVE :: H = C_NULL_PTR
      TYPE(CMAQCHEM_CFG), SAVE :: CFG
      CHARACTER(LEN=13, KIND=C_CHAR), SAVE, TARGET :: MECH = 'cb6r5_ae7_aq' // C_NULL_CHAR
      INTEGER(C_INT), SAVE, TARGET, ALLOCATABLE :: CGI( : )
      REAL, SAVE, ALLOCATABLE :: TA(:,:,:), QV(:,:,:), DENS(:,:,:), PRES(:,:,:), SEAICE(:,:), OSZ(:,:)
      TYPE(CMAQCHEM_STATS) :: ST
      CHARACTER(KIND=C_CHAR) :: MSG( 512 )
      INTEGER MIDDATE, MIDTIME, RC, N

      IF ( .NOT. C_ASSOCIATED( H ) ) THEN             ! first call, as rbdriver.F:226-371
         ALLOCATE( CGI( NUMB_MECH_SPC ), TA(NCOLS,NROWS,NLAYS), QV(NCOLS,NROWS,NLAYS),
     &             DENS(NCOLS,NROWS,NLAYS), PRES(NCOLS,NROWS,NLAYS), SEAICE(NCOLS,NROWS),
     &             OSZ(NCOLS,NROWS) )
         CGI = CGRID_INDEX
         OSZ = OCEAN + SZONE
         CFG = CMAQCHEM_CFG( C_LOC( MECH ), 0, 1, REAL( GLBL_RTOL, 8 ), REAL( GLBL_ATOL, 8 ),
     &                       NCOLS, NROWS, NLAYS, NSPCSD, C_LOC( CGI ), 0, 0 )
         RC = cmaqchem_init( CFG, H )
         IF ( RC .NE. 0 ) CALL M3EXIT( 'CHEM', JDATE, JTIME, 'cmaqchem_init failed', XSTAT1 )
      END IF
      MIDDATE = JDATE; MIDTIME = JTIME                 ! step midpoint, rbdriver.F:381-403
      CALL NEXTIME( MIDDATE, MIDTIME, SEC2TIME( TIME2SEC( TSTEP( 2 ) ) / 2 ) )
      CALL INTERPOLATE_VAR( 'SEAICE', MIDDATE, MIDTIME, SEAICE )
      CALL INTERPOLATE_VAR( 'TA',     MIDDATE, MIDTIME, TA )
      CALL INTERPOLATE_VAR( 'QV',     MIDDATE, MIDTIME, QV )
      CALL INTERPOLATE_VAR( 'DENS',   MIDDATE, MIDTIME, DENS )
      CALL INTERPOLATE_VAR( 'PRES',   MIDDATE, MIDTIME, PRES )
      CALL HETCHEM_RATES( TA, PRES, QV, CONC, DENS )   ! fills KHETERO, rbdriver.F:409
      RC = cmaqchem_step( H, CONC, TA, QV, DENS, PRES, SEAICE, OSZ, RJ, KHETERO,
     &                    JDATE, JTIME, TSTEP, ST )
      IF ( RC .NE. 0 ) THEN                            ! the reference stops the run (rbsolver.F:583)
         N = cmaqchem_last_error( MSG, INT( SIZE( MSG ), C_SIZE_T ) )
         WRITE( LOGDEV, * ) 'GPU chemistry: rc = ', RC, ' failed cells = ', ST%FAILED_CELLS
         CALL M3EXIT( 'CHEM', JDATE, JTIME, 'Convergence failure in Gas Chemistry Solver', XSTAT2 )
      END IF
      CALL HETCHEM_UPDATE_AERO( CONC )                 ! rbdriver.F:727
      END SUBROUTINE CHEM
