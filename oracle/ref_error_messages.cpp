// Recipe helper (test infrastructure only): prints the reference's own error texts.
//
// Compiled by oracle/build_ref.py (build_error_messages) against the reference's
// include/error_codes.h where it lies, into oracle/_ref/; tests/golden/make_golden.py
// runs it to write tests/golden/error_messages.npz.  One line per (code, context):
//   <code> TAB <context> TAB <getErrorMessage(code, context)>
#include <cstdio>
#include <string>

#include "error_codes.h"

int main() {
  const char* contexts[] = {"", "input validation", "symbolic evaluation backward pass", "prefix parsing"};
  // every value of the reference's enum, the unused ones between them, and values
  // outside every range
  for (long code = -1; code <= 1001; ++code) {
    const bool listed = code <= 1 || (code >= 99 && code <= 103) || (code >= 199 && code <= 206) ||
                        (code >= 299 && code <= 305) || (code >= 399 && code <= 409) ||
                        (code >= 499 && code <= 510) || code >= 999;
    if (!listed) continue;
    for (const char* ctx : contexts) {
      const std::string msg = getErrorMessage(static_cast<ErrorCode>(code), ctx);
      std::printf("%ld\t%s\t%s\n", code, ctx, msg.c_str());
    }
  }
  return 0;
}
