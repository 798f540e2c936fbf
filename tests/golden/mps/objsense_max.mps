NAME          OBJMAX
OBJSENSE
    MAX       SENSE
ROWS
 N  OBJ
 L  LIM
COLUMNS
    Y1        OBJ          2.0   LIM          1.0
    Y2        OBJ          3.0   LIM          2.0
RHS
    RHS       LIM          4.0   OBJ          1.5
BOUNDS
 UP BND       Y1           3.0
ENDATA
