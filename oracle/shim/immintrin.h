// See xmmintrin.h in this directory (test infrastructure only).
#pragma once
#include "xmmintrin.h"
