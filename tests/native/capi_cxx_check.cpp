// include/boids.h seen from C++11, the reference's own language: the
// declarations compile with warnings as errors and link as extern "C"
// symbols of libboids_gb300.so.  Nothing here touches a device: the program
// only calls entry points that check their arguments first.
#include "boids.h"

#include <cstdio>
#include <cstring>

int main()
{
    boids_params p;
    std::memset(&p, 0, sizeof p);
    p.number_of_agents = 16;
    p.field_size = 0.0;  // refused before any device work
    p.engine = BOIDS_ENGINE_GRID;
    boids_sim *sim = nullptr;
    const int rc = boids_create(&p, &sim);
    std::printf("%d %s\n", rc, boids_last_error());
    boids_destroy(sim);  // a null handle is ignored
    return rc == BOIDS_EINVAL && sim == nullptr ? 0 : 1;
}
