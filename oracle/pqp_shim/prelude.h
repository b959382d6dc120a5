/*
 * prelude.h -- force-included before each reference translation unit.  The
 * reference's C2A/LinearMath.h:538-541 defines function-like min/max macros
 * when <windows.h> has not (it always has under MSVC); pulling the standard
 * headers in first keeps those macros out of the C++ library.
 */
#include <string.h>
#include <stdlib.h>
#include <stdio.h>
#include <math.h>
#include <string>
#include <list>
#include <vector>
#include <algorithm>
#include <iostream>
#include <fstream>
