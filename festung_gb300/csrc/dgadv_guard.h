// Exception guard of the C-ABI entry points: no C++ exception crosses the boundary; a failed
// host allocation becomes DGADV_ENOMEM, any other exception DGADV_EINVAL, with the message in
// the handle's error string when there is a handle.
#pragma once
#include <exception>
#include <new>

#include "../../include/dgadv.h"

namespace dgadv {

void set_error(const dgadv_handle *h, const char *msg);   // no-op for a null handle

template <class F>
int guarded(const dgadv_handle *h, F &&f) noexcept {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    set_error(h, "host allocation failed");
    return DGADV_ENOMEM;
  } catch (const std::exception &e) {
    set_error(h, e.what());
    return DGADV_EINVAL;
  } catch (...) {
    set_error(h, "unexpected error");
    return DGADV_EINVAL;
  }
}

}  // namespace dgadv
