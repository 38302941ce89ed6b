// Fixed-memory latency histogram for the serving loop's statistics.
//
// Logarithmic bins of 0.5 % relative width from 1 microsecond up to about 18
// hours, plus the exact minimum and maximum, so a percentile is within a
// quarter of a percent of the exact order statistic however many samples a
// long-running server records.  Percentiles interpolate linearly between the
// two order statistics around rank q/100 * (count - 1), as numpy's default
// percentile does, with each order statistic represented by the geometric
// middle of its bin (clamped to the observed range); the extreme order
// statistics are the exact minimum and maximum.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace pbf_stats {

class LatencyHist {
public:
    static constexpr double kMinMs = 1e-3;
    static constexpr double kRatio = 1.005;
    static constexpr int kBins = 5000;

    LatencyHist() : bins_((size_t)kBins, 0) {}

    void add(double ms) {
        if (!(ms >= 0.0)) ms = 0.0;  // NaN and negative clock steps count as 0
        bins_[(size_t)bin_of(ms)] += 1;
        if (count_ == 0 || ms < min_) min_ = ms;
        if (count_ == 0 || ms > max_) max_ = ms;
        ++count_;
    }

    void clear() {
        std::fill(bins_.begin(), bins_.end(), 0);
        count_ = 0;
        min_ = max_ = 0.0;
    }

    uint64_t count() const { return count_; }

    double percentile(double q) const {
        if (count_ == 0) return 0.0;
        q = std::min(100.0, std::max(0.0, q));
        const double pos = q / 100.0 * (double)(count_ - 1);
        const uint64_t lo = (uint64_t)std::floor(pos);
        const uint64_t hi = std::min(lo + 1, count_ - 1);
        const double a = value_at(lo), b = value_at(hi);
        return a + (b - a) * (pos - (double)lo);
    }

    static int bin_of(double ms) {
        if (!(ms > kMinMs)) return 0;
        const double k = std::floor(std::log(ms / kMinMs) / std::log(kRatio));
        return (int)std::min<double>((double)(kBins - 1), 1.0 + std::max(0.0, k));
    }

private:
    // The k-th smallest sample (0-based), to within its bin.
    double value_at(uint64_t k) const {
        if (k == 0) return min_;
        if (k + 1 >= count_) return max_;
        uint64_t seen = 0;
        int b = 0;
        for (; b < kBins; ++b) {
            seen += bins_[(size_t)b];
            if (seen > k) break;
        }
        double v = b == 0 ? 0.0 : kMinMs * std::pow(kRatio, (double)b - 0.5);
        return std::min(max_, std::max(min_, v));
    }

    std::vector<uint64_t> bins_;
    uint64_t count_ = 0;
    double min_ = 0.0, max_ = 0.0;
};

}  // namespace pbf_stats
