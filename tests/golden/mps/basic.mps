NAME          BASIC
* a small LP with every row type
ROWS
 N  COST
 L  CAP1
 G  DEM1
 E  BAL
COLUMNS
    X1        COST         1.0   CAP1         1.0
    X1        BAL          1.0
    X2        COST         2.0   CAP1         1.0
    X2        DEM1         1.0
    X3        COST        -1.0   DEM1         1.0
    X3        BAL         -1.0
RHS
    RHS       CAP1         4.0   DEM1         1.0
    RHS       BAL          0.5
BOUNDS
 UP BND       X1           3.0
 LO BND       X2           0.5
 MI BND       X3
ENDATA
