// shim_context.cpp -- the drop-in's process-wide GPU context.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "shim_common.h"

namespace tmv {
namespace tmvg_shim {

namespace {
std::atomic<long long> g_calls{0};

void print_stats()
{
    std::fprintf(stderr, "tmvg drop-in: %lld GPU calls\n", g_calls.load());
}
}  // namespace

tmvg_handle gpu()
{
    static std::once_flag once;
    static tmvg_handle h = nullptr;
    static tmvg_status st = TMVG_OK;
    std::call_once(once, [] {
        const char* dev = std::getenv("TMVG_DEVICE");
        st = tmvg_create(&h, dev ? std::atoi(dev) : 0);
        if (std::getenv("TMVG_SHIM_STATS")) std::atexit(print_stats);
    });
    if (st != TMVG_OK) throw Error(std::string("tmvg_create: ") + tmvg_status_string(st));
    g_calls.fetch_add(1, std::memory_order_relaxed);
    return h;
}

}  // namespace tmvg_shim
}  // namespace tmv
