// Stand-in for spdlog 1.17.0 (absent offline).  poutre2 keeps its logger at level::off
// (src/base/trace.cpp:28), so a logger that drops every message is behaviour-preserving.
#pragma once
#include <memory>
#include <string>
#include "common.h"
#include "logger.h"
namespace spdlog {
inline std::shared_ptr<logger> stdout_color_st(const std::string &) { return std::make_shared<logger>(); }
inline std::shared_ptr<logger> stdout_color_mt(const std::string &) { return std::make_shared<logger>(); }
inline void shutdown() {}
}  // namespace spdlog
