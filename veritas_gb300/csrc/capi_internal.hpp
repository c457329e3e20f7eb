// Handles behind the C ABI's opaque types and the exception-to-status guard shared by
// the files that define extern "C" entry points.
#pragma once
#include <new>
#include <stdexcept>
#include <string>

#include "../../include/vx.h"
#include "engine.hpp"
#include "serve.hpp"

struct vx_ctx {
    std::unique_ptr<vx::Engine> eng;
};
struct vx_run {
    vx_ctx *ctx;
    std::unique_ptr<vx::Run> run;
};
struct vx_server {
    vx_ctx *ctx;
    std::unique_ptr<vx::Server> srv;
};

namespace vx {
extern thread_local std::string g_err;  // message of the calling thread's last failure

// Runs f, mapping exceptions to VX_ERR_* codes (the message goes to vx_last_error).
template <class F>
int guard(F &&f) {
    try {
        f();
        return VX_OK;
    } catch (const CudaError &e) {
        g_err = e.what();
        return VX_ERR_CUDA;
    } catch (const TimeoutError &e) {
        g_err = e.what();
        return VX_ERR_TIMEOUT;
    } catch (const std::invalid_argument &e) {
        g_err = e.what();
        return VX_ERR_INVALID;
    } catch (const std::bad_alloc &e) {
        g_err = e.what();
        return VX_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_err = e.what();
        return VX_ERR_STATE;
    }
}
}  // namespace vx
