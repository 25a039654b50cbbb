// DeviceMemory.hpp -- owning device allocation (DeviceMemoryManager of
// src/device/DeviceMemory.cu), over the dr_device_* calls of the C ABI, plus the
// process-wide library context the C++ interface uses.
#pragma once

#include "devilray_gb300.h"

#include <cstddef>
#include <stdexcept>
#include <string>

namespace devilray {

// The context of the C++ interface: device 0 (or DEVILRAY_DEVICE), created on
// first use and destroyed at exit.
dr_context *context();

// Throws std::runtime_error with the library's message unless status is DR_OK.
void check(dr_status status, const char *what);

}  // namespace devilray

class DeviceMemoryManager
{
public:
    DeviceMemoryManager() = default;
    ~DeviceMemoryManager() { free(); }
    DeviceMemoryManager(const DeviceMemoryManager &) = delete;
    DeviceMemoryManager &operator=(const DeviceMemoryManager &) = delete;
    DeviceMemoryManager(DeviceMemoryManager &&o) noexcept : m_ptr(o.m_ptr), m_bytes(o.m_bytes)
    {
        o.m_ptr = nullptr;
        o.m_bytes = 0;
    }
    DeviceMemoryManager &operator=(DeviceMemoryManager &&o) noexcept
    {
        if (this != &o) {
            free();
            m_ptr = o.m_ptr;
            m_bytes = o.m_bytes;
            o.m_ptr = nullptr;
            o.m_bytes = 0;
        }
        return *this;
    }

    void allocate(size_t bytes)
    {
        free();
        if (bytes == 0) return;
        devilray::check(dr_device_allocate(devilray::context(), bytes, &m_ptr), "DeviceMemoryManager::allocate");
        m_bytes = bytes;
    }
    void free()
    {
        if (m_ptr) dr_device_free(devilray::context(), m_ptr);
        m_ptr = nullptr;
        m_bytes = 0;
    }
    void copyFromHost(const void *src, size_t bytes)
    {
        if (bytes > m_bytes) throw std::runtime_error("DeviceMemoryManager::copyFromHost: beyond the allocation");
        devilray::check(dr_device_copy_from_host(devilray::context(), m_ptr, src, bytes), "copyFromHost");
    }
    void copyToHost(void *dst, size_t bytes) const
    {
        if (bytes > m_bytes) throw std::runtime_error("DeviceMemoryManager::copyToHost: beyond the allocation");
        devilray::check(dr_device_copy_to_host(devilray::context(), dst, m_ptr, bytes), "copyToHost");
    }
    template <typename T>
    T *getPtr() const { return static_cast<T *>(m_ptr); }
    bool empty() const { return m_ptr == nullptr; }
    size_t size() const { return m_bytes; }

private:
    void *m_ptr = nullptr;
    size_t m_bytes = 0;
};
