// Stand-in for spdlog 1.17.0 (see ../spdlog.h).
#pragma once
#include "../spdlog.h"
