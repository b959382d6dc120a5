/* lower-case alias used by C2A/InterpMotion.h:12 */
#include "PQP_Compile.h"
