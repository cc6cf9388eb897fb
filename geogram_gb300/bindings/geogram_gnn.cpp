// GpuNearestNeighborSearch: geogram's NearestNeighborSearch interface
// (points/nn_search.h:69-262) served by the GB300 library (include/gbv.h).
//
// A geogram maintainer compiles this file with geogram (it includes
// geogram's headers) and links it to libgbv.so, then calls
// register_gpu_nearest_neighbor_search() once -- or puts the
// geo_register_NearestNeighborSearch_creator line into GEO::initialize --
// and selects it by name: NearestNeighborSearch::create(3, "GNN"), or the
// command-line argument algo:nn_search=GNN (command_line_args.cpp:190).
//
// Threading.  geogram asks for the neighbours of stored points from
// parallel_for workers (delaunay_nn.cpp:57-70, delaunay.cpp:259-275), all on
// one search object.  Such queries are served from a batch table: the k
// nearest of every stored point, computed in one GPU call.  A table is
// immutable once published; a query that needs more neighbours than the
// current table has builds a larger one under a lock and publishes it with
// an atomic shared_ptr swap, while readers keep the table they already hold.
// Queries by coordinates go to the GPU one call at a time (a context's calls
// must not overlap), under the same lock.
#include <geogram/points/nn_search.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbv.h"

namespace GEO {

class GpuNearestNeighborSearch : public NearestNeighborSearch {
public:
    explicit GpuNearestNeighborSearch(coord_index_t dim) : NearestNeighborSearch(dim) {
        if (dim != 3 && dim != 4)
            throw std::invalid_argument("GNN: dimension must be 3 or 4");
    }

    ~GpuNearestNeighborSearch() override {
        if (ctx_ != nullptr) gbv_destroy(ctx_);
    }

    bool stride_supported() const override { return true; }

    void set_points(index_t nb_points, const double* points) override {
        set_points(nb_points, points, dimension());
    }

    void set_points(index_t nb_points, const double* points, index_t stride) override {
        std::lock_guard<std::mutex> lock(mutex_);
        // like the kd-tree (kd_tree.cpp:121-126) the object keeps the
        // caller's pointer; the GPU keeps its own copy of the points.  (Not
        // through the base class's set_points: for stride == dimension it
        // calls the two-argument overload, hence this function, again.)
        nb_points_ = nb_points;
        points_ = points;
        stride_ = stride;
        check(gbv_nn_set_points(context(), nb_points, points, dimension(), stride));
        std::atomic_store(&table_, std::shared_ptr<const Table>());
    }

    void get_nearest_neighbors(index_t k, const double* query, index_t* idx,
                               double* d2) const override {
        std::lock_guard<std::mutex> lock(mutex_);
        check(gbv_nn_get_nearest_neighbors(context(), 1, query, k, idx, d2));
    }

    void get_nearest_neighbors(index_t k, index_t q, index_t* idx, double* d2) const override {
        std::shared_ptr<const Table> t = std::atomic_load(&table_);
        if (!t || t->k < k) t = grow(k);
        std::copy_n(&t->idx[size_t(q) * t->k], k, idx);
        std::copy_n(&t->d2[size_t(q) * t->k], k, d2);
    }

private:
    struct Table {
        index_t k = 0;
        std::vector<index_t> idx;
        std::vector<double> d2;
    };

    // A table with at least k neighbours per point (at least doubling, so
    // that growing lists cost a few GPU calls), published atomically.
    std::shared_ptr<const Table> grow(index_t k) const {
        std::lock_guard<std::mutex> lock(mutex_);
        std::shared_ptr<const Table> cur = std::atomic_load(&table_);
        if (cur && cur->k >= k) return cur;  // another thread grew it meanwhile
        auto t = std::make_shared<Table>();
        t->k = std::min<index_t>(nb_points(), std::max<index_t>(k, cur ? 2 * cur->k : k));
        t->idx.resize(size_t(nb_points()) * t->k);
        t->d2.resize(size_t(nb_points()) * t->k);
        check(gbv_nn_get_nearest_neighbors_all(context(), t->k, t->idx.data(), t->d2.data()));
        std::shared_ptr<const Table> pub = t;
        std::atomic_store(&table_, pub);
        return pub;
    }

    // The GPU context, created on first use (called with mutex_ held), so
    // that creating the search object needs no GPU.
    gbv_context* context() const {
        if (ctx_ == nullptr) check(gbv_create(0, &ctx_));
        return ctx_;
    }

    static void check(gbv_status s) {
        if (s != GBV_OK) throw std::runtime_error(std::string("GNN: ") + gbv_last_error());
    }

    mutable gbv_context* ctx_ = nullptr;
    mutable std::mutex mutex_;
    mutable std::shared_ptr<const Table> table_;
};

// Registers the search under the name "GNN" (points/nn_search.h:288).
void register_gpu_nearest_neighbor_search() {
    geo_register_NearestNeighborSearch_creator(GpuNearestNeighborSearch, "GNN");
}

}  // namespace GEO
