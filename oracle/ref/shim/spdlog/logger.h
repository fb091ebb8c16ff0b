// Stand-in for spdlog 1.17.0 (see spdlog.h): every call is a no-op.
#pragma once
#include "common.h"
namespace spdlog {
class logger {
 public:
  void set_level(level::level_enum) {}
  template <class... A> void trace(A &&...) {}
  template <class... A> void debug(A &&...) {}
  template <class... A> void info(A &&...) {}
  template <class... A> void warn(A &&...) {}
  template <class... A> void error(A &&...) {}
  template <class... A> void critical(A &&...) {}
};
}  // namespace spdlog
