// Self-test of the bounded waits every tensor-core kernel of this library uses
// (umma::mbar_wait): one thread waits on an mbarrier that nothing arrives on, with a
// given limit, and reports the outcome.  It lets a test watch a wait run out without
// any copy or MMA in flight: the kernel returns, the status is readable, and the
// context stays usable.
#include "dense.cuh"

namespace gbsdf {
namespace {

// status[0] = 1 when the wait ran out, 0 when the barrier completed; status[1] = the
// elapsed wall time in microseconds (clamped to int)
__global__ void k_selftest_wait(uint64_t timeout_ns, int arrive_first, int* status) {
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x != 0) return;
    umma::mbar_init(&mbar, 1);
    umma::fence_mbar_init();
    if (arrive_first) umma::mbar_arrive(&mbar);
    const uint64_t t0 = umma::global_timer_ns();
    const bool done = umma::mbar_wait(&mbar, 0u, timeout_ns);
    const uint64_t us = (umma::global_timer_ns() - t0) / 1000u;
    status[0] = done ? 0 : 1;
    status[1] = (int)(us > 0x7fffffffu ? 0x7fffffffu : us);
}

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_selftest_wait(int64_t timeout_ns, int arrive_first, int* status, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(status != nullptr, "NULL status");
    GBSDF_CHECK_ARG(timeout_ns >= 0 && timeout_ns <= 2000000000LL, "timeout %lld ns: 0 to 2 s", (long long)timeout_ns);
    k_selftest_wait<<<1, 32, 0, as_stream(stream)>>>((uint64_t)timeout_ns, arrive_first ? 1 : 0, status);
    return launch_status("selftest_wait");
}
