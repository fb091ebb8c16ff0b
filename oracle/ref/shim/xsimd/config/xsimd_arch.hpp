// Stand-in for xsimd 14.2.0's arch header (absent offline); see ../xsimd.hpp.
#pragma once
#include "../xsimd.hpp"
