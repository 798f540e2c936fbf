NAME          NONROW
ROWS
 L  FIRST
 G  SECOND
 E  THIRD
COLUMNS
    U         FIRST        2.0   SECOND       1.0
    V         FIRST        1.0   THIRD        1.0
    V         SECOND       3.0
RHS
    RHS       SECOND       1.0   THIRD        2.0
    RHS       FIRST        5.0
ENDATA
