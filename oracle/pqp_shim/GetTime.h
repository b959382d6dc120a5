/* GetTime.h -- PQP-interface restatement: wall-clock seconds. */
#ifndef C2A_SHIM_GETTIME_H
#define C2A_SHIM_GETTIME_H
double GetTime();
#endif
