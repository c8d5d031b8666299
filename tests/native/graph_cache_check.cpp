// CPU check of the graph cache's invalidation logic (capsp::GraphCache).
// A fake graph handle records whether it was destroyed; the sequence mirrors
// a handle that captures a 4-RHS solve, grows its scratch for a 16-RHS solve
// (which frees what the capture points at) and is asked for the 4-RHS graph again.
#include "graph_cache.h"

#include <cstdio>
#include <cstdlib>
#include <set>

static std::set<int> g_live;
static int g_destroyed = 0;

static void destroy_fake(int e)
{
    if (!g_live.erase(e)) {
        std::printf("FAIL: graph %d destroyed twice or never created\n", e);
        std::exit(1);
    }
    ++g_destroyed;
}

typedef capsp::GraphCache<int, destroy_fake> Cache;

static int g_next = 1;
static int make_graph()
{
    g_live.insert(g_next);
    return g_next++;
}

#define CHECK(c)                                                       \
    do {                                                               \
        if (!(c)) {                                                    \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);           \
            return 1;                                                  \
        }                                                              \
    } while (0)

static capsp::GraphKey key(const Cache &c, int nrhs, int block = 256)
{
    static double b[64], x[64];
    return capsp::GraphKey{b, x, nrhs, nrhs, (const void *)0x10, 1, 1, block, 1, 32, 1, c.generation()};
}

int main()
{
    {
        Cache c;
        // capture k = 4, replay hits
        const capsp::GraphKey k4 = key(c, 4);
        CHECK(c.find(k4) == nullptr);
        CHECK(c.put(k4, make_graph()));
        CHECK(c.size() == 1 && c.find(k4) != nullptr);
        // a different launch shape is a different graph, not a hit
        CHECK(c.find(key(c, 4, 128)) == nullptr);
        // k = 16 grows the scratch: the handle invalidates
        c.invalidate();
        CHECK(c.size() == 0 && g_destroyed == 1 && g_live.empty());
        // the old key (old generation) never hits again, and cannot be re-inserted
        CHECK(c.find(k4) == nullptr);
        const int stale = make_graph();
        CHECK(!c.put(k4, stale));
        CHECK(g_live.count(stale) == 0 && c.size() == 0);
        // the k = 4 solve recaptures under the new generation
        const capsp::GraphKey k4b = key(c, 4);
        CHECK(!(k4b.tie() == k4.tie()));
        CHECK(c.find(k4b) == nullptr);
        CHECK(c.put(k4b, make_graph()));
        CHECK(c.find(k4b) != nullptr && c.size() == 1);
        // replacing an entry destroys the old graph
        const int before = g_destroyed;
        CHECK(c.put(k4b, make_graph()));
        CHECK(g_destroyed == before + 1 && c.size() == 1);
        CHECK(c.put(key(c, 16), make_graph()));
        CHECK(c.size() == 2);
    }
    // the cache's destruction (handle teardown) frees every graph
    CHECK(g_live.empty());
    std::printf("graph cache ok: %d graphs destroyed\n", g_destroyed);
    return 0;
}
