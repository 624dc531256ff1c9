// ORACLE — test infrastructure only.
//
// C entry points around the reference's own greedy colouring, compiled together with
// spg/source/utils/graphColoring.cpp from the reference checkout (see oracle/build.py). The
// reference functions are called unmodified: coloring::colorVertices (graphColoring.cpp:72-84)
// and coloring::colorStencils (graphColoring.cpp:51-70).
#include <spg/utils/graphColoring.h>

#include <exception>
#include <vector>

extern "C" {

// sets: nSets flat stencil arrays, entries[s] of length counts[s], with stencil sizes sizes[s].
int ref_color_vertices(int nVertices, int nSets, const int *sizes, const int *counts, const int *const *entries,
                       int *out)
{
    try {
        std::vector<spg::coloring::FlatStencils> sets;
        for (int s = 0; s < nSets; ++s) {
            spg::coloring::FlatStencils f;
            f.entries.assign(entries[s], entries[s] + counts[s]);
            f.stencilSize = sizes[s];
            sets.push_back(std::move(f));
        }
        const auto colors = spg::coloring::colorVertices(nVertices, sets);
        for (size_t i = 0; i < colors.size(); ++i) out[i] = colors[i];
        return 0;
    } catch (const std::exception &) {
        return 1;
    }
}

int ref_color_stencils(int stencilSize, int count, const int *entries, int *out)
{
    try {
        spg::coloring::FlatStencils f;
        f.entries.assign(entries, entries + count);
        f.stencilSize = stencilSize;
        const auto colors = spg::coloring::colorStencils(f);
        for (size_t i = 0; i < colors.size(); ++i) out[i] = colors[i];
        return 0;
    } catch (const std::exception &) {
        return 1;
    }
}
}
