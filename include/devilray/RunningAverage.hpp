// RunningAverage.hpp -- mean of the last N samples (include/RunningAverage.hpp).
#pragma once

#include <deque>
#include <numeric>

struct RunningAverage
{
    explicit RunningAverage(int sampleCount) : m_sampleCount(sampleCount) {}

    void add(double value)
    {
        m_samples.push_back(value);
        if ((int)m_samples.size() > m_sampleCount) m_samples.pop_front();
    }
    double mean() const
    {
        return m_samples.empty() ? 0.0 : std::accumulate(m_samples.begin(), m_samples.end(), 0.0) / m_samples.size();
    }
    void reset() { m_samples.clear(); }

private:
    std::deque<double> m_samples;
    int m_sampleCount;
};
