// The C++ mirror's Deck over ogs_deck_* (host code, no GPU): reads the deck
// given on the command line and prints the mesh size and the Dirichlet rows
// of its GROUNDWATER_FLOW conditions.
#include <cstdio>

#include "ogs_gpu.hpp"

int main(int argc, char** argv)
{
    if (argc < 4) return 2;
    try
    {
        ogs_gpu::Deck deck(argv[1], argv[2], argv[3]);
        const ogs_mesh_desc d = deck.mesh_desc();
        const auto bc = deck.dirichlet("GROUNDWATER_FLOW", "HEAD");
        std::printf("nodes %lld elements %lld type %d h %.6f bc %zu\n", (long long)d.n_nodes,
                    (long long)d.n_elements, d.elem_type, deck.min_edge_length(), bc.size());
        for (const auto& rv : bc) std::printf("%lld %.17g\n", (long long)rv.first, rv.second);
    }
    catch (const ogs_gpu::Error& e)
    {
        std::printf("error %d %s\n", (int)e.status, e.what());
        return 1;
    }
    return 0;
}
