// A stand-in for the nanoflann k-d tree with the one query the reference's
// PointsTensor adapter makes (core/include/kdtree_tensor.hpp: knnSearch of
// the k nearest points under L2_Simple_Adaptor), so that adapter compiles
// unchanged here, where nanoflann is not installed — TEST INFRASTRUCTURE
// ONLY.  nanoflann's knnSearch returns the exact k nearest points in
// ascending squared distance; L2_Simple_Adaptor accumulates (query - point)
// squared per dimension in the distance type.  This does the same by brute
// force (ties in index order).
#pragma once

#include <algorithm>
#include <cstddef>
#include <utility>
#include <vector>

namespace nanoflann {

struct KDTreeSingleIndexAdaptorParams {
    size_t leaf_max_size;
    KDTreeSingleIndexAdaptorParams(size_t leaf = 10) : leaf_max_size(leaf) {}
};

template <class T, class DataSource, class DistanceType = T> struct L2_Simple_Adaptor {
    const DataSource &data_source;
    explicit L2_Simple_Adaptor(const DataSource &d) : data_source(d) {}
    DistanceType evalMetric(const T *a, size_t b_idx, size_t size) const {
        DistanceType result = DistanceType();
        for (size_t i = 0; i < size; ++i) {
            const DistanceType diff = a[i] - data_source.kdtree_get_pt(b_idx, i);
            result += diff * diff;
        }
        return result;
    }
};

template <class Distance, class DatasetAdaptor, int DIM = -1, class IndexType = size_t>
class KDTreeSingleIndexAdaptor {
public:
    KDTreeSingleIndexAdaptor(int dims, const DatasetAdaptor &ds,
                             const KDTreeSingleIndexAdaptorParams &params = KDTreeSingleIndexAdaptorParams())
        : dims_(dims), ds_(ds), metric_(ds) {
        (void)params;
    }
    template <class T, class D>
    size_t knnSearch(const T *query, size_t k, IndexType *out_indices, D *out_dists) const {
        const size_t n = ds_.kdtree_get_point_count();
        std::vector<std::pair<D, size_t>> all(n);
        for (size_t i = 0; i < n; i++) all[i] = {metric_.evalMetric(query, i, (size_t)dims_), i};
        const size_t m = std::min(k, n);
        std::partial_sort(all.begin(), all.begin() + (long)m, all.end());
        for (size_t j = 0; j < m; j++) {
            out_indices[j] = (IndexType)all[j].second;
            out_dists[j] = all[j].first;
        }
        return m;
    }

private:
    int dims_;
    const DatasetAdaptor &ds_;
    Distance metric_;
};

}  // namespace nanoflann
