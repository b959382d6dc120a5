/* case alias: C2A/InterpMotion.h:13 includes "C2A/c2a_bv.h" */
#include <C2A/C2A_BV.h>
