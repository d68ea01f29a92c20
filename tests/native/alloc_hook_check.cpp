// Drives rfba::DevBuf (rfba_gb300/csrc/devbuf.h) with RFBA_TEST_ALLOC_FAIL set
// and prints one line per allocation: "<status> <error text>". Built and run by
// tests/test_alloc_failure_cpu.py. On a machine without a GPU every real
// cudaMalloc fails with a CUDA error, which is what the other allocations show
// there; the injected one must report RFBA_ERR_NOMEM with the buffer's name.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "../../rfba_gb300/csrc/devbuf.h"

namespace rfba {
static std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
}  // namespace rfba

int main(int argc, char** argv) {
    // argv[1]: value for RFBA_TEST_ALLOC_FAIL; argv[2]: allocations to make
    if (argc < 3) return 2;
    setenv("RFBA_TEST_ALLOC_FAIL", argv[1], 1);
    const int n = std::atoi(argv[2]);
    for (int i = 0; i < n; ++i) {
        rfba::DevBuf b;
        const std::string name = "buffer " + std::to_string(i + 1);
        rfba::g_err.clear();
        const int s = b.ensure(1024, name.c_str());
        std::printf("%d %s\n", s, rfba::g_err.c_str());
        b.release();
    }
    return 0;
}
