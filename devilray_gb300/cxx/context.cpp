// context.cpp -- the library context of the C++ interface.
#include "device/DeviceMemory.hpp"

#include <cstdlib>
#include <mutex>

namespace devilray {
namespace {

struct Holder {
    dr_context *ctx = nullptr;
    ~Holder()
    {
        if (ctx) dr_context_destroy(ctx);
    }
};

}  // namespace

dr_context *context()
{
    static Holder holder;
    static std::once_flag once;
    static dr_status status = DR_OK;
    std::call_once(once, [] {
        dr_context_config cfg{};
        const char *dev = std::getenv("DEVILRAY_DEVICE");
        cfg.device = dev ? std::atoi(dev) : 0;
        status = dr_context_create(&cfg, &holder.ctx);
    });
    check(status, "devilray::context");
    return holder.ctx;
}

void check(dr_status status, const char *what)
{
    if (status == DR_OK) return;
    const char *msg = dr_last_error_string();
    throw std::runtime_error(std::string(what) + ": " + (msg ? msg : "error") + " (status " +
                             std::to_string((int)status) + ")");
}

}  // namespace devilray
