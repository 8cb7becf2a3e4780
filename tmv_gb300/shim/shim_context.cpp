// shim_context.cpp -- the drop-in's process-wide GPU context.
#include <cstdlib>
#include <mutex>

#include "shim_common.h"

namespace tmv {
namespace tmvg_shim {

tmvg_handle gpu()
{
    static std::once_flag once;
    static tmvg_handle h = nullptr;
    static tmvg_status st = TMVG_OK;
    std::call_once(once, [] {
        const char* dev = std::getenv("TMVG_DEVICE");
        st = tmvg_create(&h, dev ? std::atoi(dev) : 0);
    });
    if (st != TMVG_OK) throw Error(std::string("tmvg_create: ") + tmvg_status_string(st));
    return h;
}

}  // namespace tmvg_shim
}  // namespace tmv
