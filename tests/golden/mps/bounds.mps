NAME          BOUNDKINDS
ROWS
 N  OBJ
 L  C1
COLUMNS
    P1        OBJ          1.0   C1           1.0
    P2        OBJ          1.0   C1           1.0
    P3        OBJ          1.0   C1           1.0
    P4        OBJ          1.0   C1           1.0
    P5        OBJ          1.0   C1           1.0
    P6        OBJ          1.0   C1           1.0
    P7        OBJ          1.0   C1           1.0
    P8        OBJ          1.0   C1           1.0
RHS
    RHS       C1           100.0
BOUNDS
 FX BND       P1           4.0
 BV BND       P2
 PL BND       P3
 MI BND       P4
 UP BND       P4           -1.0
 LO BND       P5           -3.0
 UP BND       P6           -2.5
 FR BND       P7
 LI BND       P8           2.0
 UP BND       GHOST        1.0
ENDATA
