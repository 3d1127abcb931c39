// Driver of tests/test_sanitizers_cpu.py: runs the library's host-side parsers
// of untrusted input -- FLINT's table files (flint::tables_read: Tecplot ASCII
// and SZL binary) and the mechanism IR blob (flint::ir_parse) -- on the files
// named on the command line, in a build instrumented by AddressSanitizer and
// UndefinedBehaviorSanitizer.  It makes no CUDA call, so it runs without a GPU.
//
//   sanitize_host_parsers --tables <folder> <prefix> ... --ir <blob file> ...
//
// Prints one line per input with the parser's return code; any memory or
// undefined-behaviour error is reported by the sanitizers and ends the run.
#include <cstdio>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "../flint_gb300/csrc/flint_host.h"

int main(int argc, char** argv) {
  int inputs = 0;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--tables" && i + 2 < argc) {
      flint_table_set_s t;
      std::string err;
      const int rc = flint::tables_read(argv[i + 1], argv[i + 2], &t, err);
      std::printf("tables %s %s rc=%d ns=%d %s\n", argv[i + 1], argv[i + 2], rc, t.ns, err.c_str());
      i += 2;
      ++inputs;
    } else if (a == "--ir" && i + 1 < argc) {
      std::ifstream f(argv[i + 1], std::ios::binary);
      std::vector<char> blob((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
      flint_ir_s ir;
      std::string err;
      const int rc = flint::ir_parse(blob.empty() ? nullptr : blob.data(), (int64_t)blob.size(), &ir, err);
      std::printf("ir %s bytes=%zu rc=%d ns=%d nr=%d %s\n", argv[i + 1], blob.size(), rc, ir.ns, ir.nr, err.c_str());
      i += 1;
      ++inputs;
    } else {
      std::fprintf(stderr, "bad argument %s\n", argv[i]);
      return 2;
    }
  }
  std::printf("inputs %d\n", inputs);
  return 0;
}
