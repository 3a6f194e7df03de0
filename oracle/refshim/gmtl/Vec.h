// GMTL header name used by the reference sources; the shim is one file.
#pragma once
#include "shim.h"
