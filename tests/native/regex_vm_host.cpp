// Host build of the REGEXP_REPLACE compiler and matcher (the same sources the
// string pre-pass compiles for the device), for tests that compare it with
// Python's re on many patterns without a GPU.  Built by tests/test_regex.py.
#include <cstring>
#include <string>

#include "regex.cpp"
#include "regex_vm.h"

extern "C" int gx_test_regex_replace(const char* pattern, const char* repl, const char* subject, int n, int keep,
                                     char* out, int cap, char* err, int err_len) {
  std::string program, tmpl;
  try {
    gx::compile_regex_replace(pattern, repl, &program, &tmpl);
  } catch (const gx::Error& e) {
    std::snprintf(err, (size_t)err_len, "%s", e.what());
    return -1 - (int)e.code;
  }
  const unsigned char* p = (const unsigned char*)subject;
  const int len = gx::regex_replace_row((const unsigned char*)program.data(), (const unsigned char*)tmpl.data(),
                                        (int)tmpl.size(), p, n, keep, nullptr);
  if (len > cap) return len;
  gx::regex_replace_row((const unsigned char*)program.data(), (const unsigned char*)tmpl.data(), (int)tmpl.size(), p,
                        n, keep, (unsigned char*)out);
  return len;
}
