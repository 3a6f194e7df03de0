// Force-included (-include) before every reference source that
// oracle/build_ref.py compiles for the ray-tracing pin.  It pulls in the
// standard headers those sources use, then routes their pow / powf calls
// to the portable power function the oracle and the CUDA path share (the
// documented substitution for libm's pow, whose last-ulp results differ
// between C libraries).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

extern "C" float ear_ref_powf(float x, float y);
#define pow(x, y) ear_ref_powf((float)(x), (float)(y))
#define powf(x, y) ear_ref_powf((float)(x), (float)(y))
