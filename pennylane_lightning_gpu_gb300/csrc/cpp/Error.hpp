// Exceptions and abort macros of the drop-in C++ layer.  Same names and
// message style as the pennylane-lightning Error.hpp that the reference
// includes (PL_ABORT / PL_ABORT_IF / PL_ABORT_IF_NOT / PL_ASSERT and
// LightningException, registered in Python as PLException at
// Bindings.cpp:1734).
#pragma once

#include <exception>
#include <string>
#include <utility>

#include "lgpu.h"

namespace Pennylane::Util {

class LightningException : public std::exception {
  private:
    std::string err_msg;

  public:
    explicit LightningException(std::string err_msg) noexcept : err_msg{std::move(err_msg)} {}
    LightningException(const LightningException &) = default;
    LightningException(LightningException &&) noexcept = default;
    LightningException &operator=(const LightningException &) = default;
    LightningException &operator=(LightningException &&) noexcept = default;
    ~LightningException() override = default;
    [[nodiscard]] auto what() const noexcept -> const char * override { return err_msg.c_str(); }
};

[[noreturn]] inline void Abort(const char *message, const char *file_name, int line, const char *function_name) {
    std::string msg = std::string("[") + file_name + "][Line:" + std::to_string(line) + "][Method:" +
                      function_name + "]: Error in PennyLane Lightning: " + message;
    throw LightningException(msg);
}

// Convert an lgpu status into a LightningException carrying the library's message.
inline void check_lgpu(lgpu_status_t st, const char *what) {
    if (st != LGPU_OK) {
        std::string msg = std::string(what) + ": " + lgpu_last_error_string();
        throw LightningException(msg);
    }
}

} // namespace Pennylane::Util

#define PL_ABORT(message) Pennylane::Util::Abort(message, __FILE__, __LINE__, __func__)
#define PL_ABORT_IF(expression, message)                                                                \
    if ((expression)) {                                                                                \
        PL_ABORT(message);                                                                             \
    }
#define PL_ABORT_IF_NOT(expression, message)                                                            \
    if (!(expression)) {                                                                               \
        PL_ABORT(message);                                                                             \
    }
#define PL_ASSERT(expression) PL_ABORT_IF_NOT(expression, "Assertion failed: " #expression)
#define PL_LGPU_IS_SUCCESS(expr) Pennylane::Util::check_lgpu((expr), #expr)

namespace Pennylane {
using Util::LightningException;
}
