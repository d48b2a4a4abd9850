// Shared error state of the C ABI (dg_last_error).
#pragma once
#include <exception>
#include <new>
#include <string>

#include "../../../include/dgcuda.h"

namespace dg {
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

// Runs an entry point's body so that no exception crosses the C ABI: host
// allocation failures become DG_ERR_NOMEM, other exceptions DG_ERR_ARG.
template <typename F>
int guarded(F &&body) {
    try {
        return body();
    } catch (const std::bad_alloc &) {
        return fail(DG_ERR_NOMEM, "out of host memory");
    } catch (const std::exception &e) {
        return fail(DG_ERR_ARG, e.what());
    }
}
}  // namespace dg
