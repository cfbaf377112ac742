// C++ side of the pgx C ABI for pagmo users: status codes become the
// exceptions pagmo itself throws, and one context per device is shared by
// every adaptor object (pagmo copies UDPs and UDBFEs freely).
#ifndef PAGMO_GB300_PGX_HPP
#define PAGMO_GB300_PGX_HPP

#include <array>
#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

#include <pagmo/exceptions.hpp>

#include "../pgx.h"

namespace pagmo_gb300
{

// PGX_ERR_INVALID -> std::invalid_argument (pagmo_throw(std::invalid_argument, ...)),
// PGX_ERR_NOTIMPL -> pagmo::not_implemented_error, PGX_ERR_CAPACITY ->
// std::overflow_error, anything else -> std::runtime_error.
inline void check(int status)
{
    if (status == PGX_OK) return;
    const std::string msg = pgx_last_error();
    if (status == PGX_ERR_INVALID) throw std::invalid_argument(msg);
    if (status == PGX_ERR_NOTIMPL) throw pagmo::not_implemented_error(msg);
    if (status == PGX_ERR_CAPACITY) throw std::overflow_error(msg);
    throw std::runtime_error(msg.empty() ? "pgx error " + std::to_string(status) : msg);
}

// The process-wide context of a device, created on first use and released
// at exit. Calls on it are serialised inside the library.
inline pgx_context *device_context(int device = 0)
{
    struct holder {
        std::once_flag once;
        pgx_context *ctx = nullptr;
        int status = PGX_OK;
        std::string error;
        ~holder()
        {
            if (ctx) pgx_context_destroy(ctx);
        }
    };
    static std::array<holder, 64> slots;
    if (device < 0 || device >= static_cast<int>(slots.size())) throw std::invalid_argument("device ordinal out of range");
    holder &h = slots[static_cast<size_t>(device)];
    std::call_once(h.once, [&h, device]() {
        h.status = pgx_context_create(device, &h.ctx);
        if (h.status != PGX_OK) h.error = pgx_last_error();
    });
    if (h.status != PGX_OK) {
        if (h.status == PGX_ERR_INVALID) throw std::invalid_argument(h.error);
        throw std::runtime_error(h.error);
    }
    return h.ctx;
}

} // namespace pagmo_gb300

#endif
