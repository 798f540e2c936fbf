NAME          RANGESMAX
OBJSENSE
    MAXIMIZE
ROWS
 G  R1
 N  PROFIT
 L  R2
 E  R3
 N  OTHER
 E  R4
 G  R5
COLUMNS
    A         PROFIT       3.0   R1           1.0
    A         R2           2.0   OTHER        9.0
    MARKER                 'MARKER'                 'INTORG'
    B         PROFIT       1.0   R1           1.0
    B         R3           1.0   NOSUCH       5.0
    R2        4.0
    B         PROFIT       0.5
    MARKER                 'MARKER'                 'INTEND'
    C         R4           2.0   R5           1.0
    C         R2           1.0   R2           1.0
RHS
    RHS       R1           1.0   R2           8.0
    RHS       R3           2.0   R4           3.0
    RHS       R5           0.5   PROFIT      -7.0
RANGES
    RNG       R1           2.5   R2          -3.0
    RNG       R3           1.5   R4          -2.0
    RNG       R5          -1.0
BOUNDS
 UP BND       A            10.0
 LO BND       C            -2.0
 UP BND       C            6.0
ENDATA
