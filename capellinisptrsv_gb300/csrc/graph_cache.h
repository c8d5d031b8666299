// Cache of instantiated CUDA graphs of one solver handle (host-only logic).
//
// A captured solve bakes in device pointers (the publication scratch, the
// sum-and-count words, the value arrays, the selector table) and settings (the
// launch shape, the wait budget, the debug hooks).  The cache therefore keys
// every graph on the caller's vectors and launch parameters *and* on a
// generation number that the handle bumps whenever any of that baked-in state
// changes; bumping also destroys every cached graph at once, so a graph that
// references freed scratch is never replayed and never kept.
//
// The Exec type and its destroy function are template parameters so that the
// logic compiles and is tested without the CUDA runtime.
#pragma once

#include <cstdint>
#include <map>
#include <tuple>

namespace capsp {

// Launch parameters of a captured solve besides the generation number.
struct GraphKey {
    const void *b;
    const void *x;
    int nrhs;
    int64_t ld;
    const void *stream;
    int kind, rows_per_thread, block, blocks_per_sm, border, dflt;
    unsigned long long gen;

    auto tie() const
    {
        return std::tie(b, x, nrhs, ld, stream, kind, rows_per_thread, block, blocks_per_sm, border, dflt, gen);
    }
    bool operator<(const GraphKey &o) const { return tie() < o.tie(); }
};

template <typename Exec, void (*Destroy)(Exec)>
class GraphCache {
public:
    GraphCache() = default;
    GraphCache(const GraphCache &) = delete;
    GraphCache &operator=(const GraphCache &) = delete;
    ~GraphCache() { clear(); }

    // generation that a key built now must carry
    unsigned long long generation() const { return gen_; }

    // Something a captured graph depends on changed (scratch reallocated,
    // values re-pointed, a setting altered): every cached graph is destroyed.
    void invalidate()
    {
        ++gen_;
        clear();
    }

    // cached graph for the key, or nullptr; a key of an older generation never hits
    Exec *find(const GraphKey &k)
    {
        if (k.gen != gen_)
            return nullptr;
        auto it = map_.find(k);
        return it == map_.end() ? nullptr : &it->second;
    }

    // takes ownership of e; returns false (and destroys e) for a stale key
    bool put(const GraphKey &k, Exec e)
    {
        if (k.gen != gen_) {
            Destroy(e);
            return false;
        }
        auto it = map_.find(k);
        if (it != map_.end()) {
            Destroy(it->second);
            it->second = e;
        } else {
            map_.emplace(k, e);
        }
        return true;
    }

    size_t size() const { return map_.size(); }

    void clear()
    {
        for (auto &kv : map_)
            Destroy(kv.second);
        map_.clear();
    }

private:
    std::map<GraphKey, Exec> map_;
    unsigned long long gen_ = 0;
};

}  // namespace capsp
