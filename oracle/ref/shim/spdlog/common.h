// Stand-in for spdlog 1.17.0 (see spdlog.h).
#pragma once
namespace spdlog { namespace level { enum level_enum { trace, debug, info, warn, err, critical, off }; } }
