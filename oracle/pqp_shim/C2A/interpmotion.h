/* case alias: C2A/src/InterpMotion.cpp:1 includes "C2A/interpmotion.h" */
#include <C2A/InterpMotion.h>
