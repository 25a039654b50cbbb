// Vector.hpp -- growable host vector with a lazily refreshed device copy
// (DeviceVector of include/device/Vector.hpp). Move-only; no default
// constructor (construct from a std::vector, e.g. `DeviceVector<T> v{{}}`).
#pragma once

#include "device/DeviceMemory.hpp"

#include <span>
#include <vector>

template <typename T>
struct DeviceVector
{
    explicit DeviceVector(std::vector<T> data) : m_host(std::move(data)) {}
    DeviceVector() = delete;

    void deleteDeviceMemory()
    {
        m_device.free();
        m_deviceNeedsUpdate = true;
    }
    void ensureDeviceAllocation()
    {
        if (m_deviceNeedsUpdate) {
            m_device.allocate(sizeof(T) * size());
            updateDeviceData();
            m_deviceNeedsUpdate = false;
        }
    }
    void updateDeviceData()
    {
        if (size() > 0) m_device.copyFromHost(m_host.data(), sizeof(T) * size());
    }
    void push_back(T elem)
    {
        m_host.push_back(std::move(elem));
        m_deviceNeedsUpdate = true;
    }

    T *devicePtr() { return m_device.template getPtr<T>(); }
    std::span<T> deviceSpan() { return std::span{devicePtr(), size()}; }
    T *hostPtr() { return m_host.data(); }
    const T *hostPtr() const { return m_host.data(); }
    std::span<T> hostSpan() { return std::span{m_host.data(), size()}; }
    std::span<const T> hostSpan() const { return std::span{m_host.data(), size()}; }
    T &operator[](size_t i) { return m_host[i]; }
    const T &operator[](size_t i) const { return m_host[i]; }
    size_t size() const { return m_host.size(); }

private:
    std::vector<T> m_host;
    DeviceMemoryManager m_device;
    bool m_deviceNeedsUpdate = true;
};
