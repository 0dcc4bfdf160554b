// Shared host-side definitions of the GB300 HEOM library.
#pragma once
#include <complex>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/heom_gb300.h"

namespace heom {

using cd = std::complex<double>;

constexpr double kHbar = 0.658211928;     // meV ps (reference include/sizes:23)
constexpr double kPi = 3.141592653589793238;
constexpr double kJconst = 1.602177e5;    // current unit factor (reference include/sizes:27)
constexpr double kDsmall = 1e-32;         // zero test of the reference (include/sizes:34)

void set_error(const std::string &msg);

struct HeomError {
    int code;
    std::string msg;
};
[[noreturn]] void fail(int code, const std::string &msg);

// Run a callable and translate exceptions into an error code + message.
template <class F>
int guarded(F &&f) {
    try {
        f();
        return HEOM_OK;
    } catch (const HeomError &e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc &) {
        set_error("host allocation failed");
        return HEOM_E_NOMEM;
    } catch (const std::exception &e) {
        set_error(e.what());
        return HEOM_E_ARG;
    }
}

}  // namespace heom
