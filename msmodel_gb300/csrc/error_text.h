// error_text.h -- the library's error text (msgpu_last_error), for every
// translation unit, CUDA or host-only.
#pragma once

namespace msg {

// sets the text msgpu_last_error returns and passes `code` through
int record_error(int code, const char* what);

}  // namespace msg
