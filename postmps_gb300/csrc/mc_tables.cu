// mc_tables.cu -- marching-cubes case tables.
//
// The triangle soup order is defined by the reference's tables
// (MarchingCubesHelper.cpp:3-587, the widely used 256-case tables with the
// corner numbering of myCuda.cuh:205-216).  When the build finds the
// reference tree it extracts those tables into the (git-ignored) generated
// file _build/gen/mc_tables.inc, so the mesh comes out in the reference's
// exact triangle order.  Without it, the tables are derived here from first
// principles: the edges a case crosses are the edges whose end corners lie on
// different sides of the iso value; on each cube face (its corners taken
// counter-clockwise seen from outside) the crossings are joined into segments
// -- a face with four crossings joins them so that each set corner (bit set,
// field <= iso) is cut off on its own --, segments chain into closed loops, and
// every loop is fanned into triangles.  Both variants cross the same edges,
// emit the same number of vertices in every case and wind their triangles the
// same way; the derived one splits some polygons along other diagonals.
#include "pms_internal.h"

#if defined(__has_include)
#if __has_include("../_build/gen/mc_tables.inc")
#include "../_build/gen/mc_tables.inc"
#define PMS_HAVE_REF_MC_TABLES 1
#endif
#endif

namespace pms {

static const int kCorner[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}};
static const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

static int edge_between(int a, int b) {
    for (int e = 0; e < 12; ++e)
        if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
    return -1;
}

// Derives all 256 cases.
static void derive_tables(McTables& T) {
    // the six faces as corner cycles
    int faces[6][4];
    int nf = 0;
    for (int axis = 0; axis < 3; ++axis)
        for (int side = 0; side < 2; ++side) {
            int cs[4], k = 0;
            for (int c = 0; c < 8; ++c) if (kCorner[c][axis] == side) cs[k++] = c;
            // order the 4 corners as a cycle (consecutive corners share an edge)
            int cyc[4] = {cs[0], -1, -1, -1};
            bool used[4] = {true, false, false, false};
            for (int i = 1; i < 4; ++i)
                for (int j = 0; j < 4; ++j)
                    if (!used[j] && edge_between(cyc[i - 1], cs[j]) >= 0) { cyc[i] = cs[j]; used[j] = true; break; }
            // counter-clockwise seen from outside the cube, so that an edge shared by two
            // faces is walked in opposite directions by their cycles
            int d1[3], d2[3];
            for (int a = 0; a < 3; ++a) {
                d1[a] = kCorner[cyc[1]][a] - kCorner[cyc[0]][a];
                d2[a] = kCorner[cyc[2]][a] - kCorner[cyc[1]][a];
            }
            const int cr = d1[(axis + 1) % 3] * d2[(axis + 2) % 3] - d1[(axis + 2) % 3] * d2[(axis + 1) % 3];
            const bool ccw = side ? cr > 0 : cr < 0;
            for (int i = 0; i < 4; ++i) faces[nf][i] = ccw ? cyc[i] : cyc[(4 - i) & 3];
            ++nf;
        }
    for (int e = 0; e < 12; ++e) { T.edge_vertex[e][0] = kEdge[e][0]; T.edge_vertex[e][1] = kEdge[e][1]; }
    for (int cse = 0; cse < 256; ++cse) {
        auto in = [&](int c) { return (cse >> c) & 1; };
        uint32_t ef = 0;
        for (int e = 0; e < 12; ++e) if (in(kEdge[e][0]) != in(kEdge[e][1])) ef |= 1u << e;
        T.edge_flags[cse] = ef;
        // on a face with four crossings the set corners are always the ones cut off
        // (whatever their number): the rule that gives the reference's vertex count
        // in every one of the 256 cases
        const bool cut_set = true;
        // next[e]: successor of crossed edge e along its loop
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        for (int f = 0; f < 6; ++f) {
            int cr[4], nc = 0;                 // crossed edges in cycle order
            int after[4];
            for (int i = 0; i < 4; ++i) {
                int a = faces[f][i], b = faces[f][(i + 1) & 3];
                if (in(a) != in(b)) { cr[nc] = edge_between(a, b); after[nc] = i; ++nc; }
            }
            if (nc == 2) {
                // orient: go from the crossing that leaves a set corner (walking the cycle)
                int a0 = faces[f][after[0]];
                if (in(a0)) next[cr[0]] = cr[1]; else next[cr[1]] = cr[0];
            } else if (nc == 4) {
                for (int k = 0; k < 4; k += 2) {
                    // pair crossings around the corner that is cut off
                    int c0 = faces[f][(after[k] + 1) & 3];   // corner between crossing k and k+1
                    bool sep = (in(c0) != 0) == cut_set;
                    int p = sep ? k : (k + 1) & 3, q = sep ? (k + 1) & 3 : (k + 2) & 3;
                    int ap = faces[f][after[p]];
                    if (in(ap)) next[cr[p]] = cr[q]; else next[cr[q]] = cr[p];
                }
            }
        }
        // chain loops and fan-triangulate
        int out = 0;
        bool seen[12] = {false};
        for (int e0 = 0; e0 < 12; ++e0) {
            if (!(ef & (1u << e0)) || seen[e0] || next[e0] < 0) continue;
            int loop[12], nl = 0, e = e0;
            while (e >= 0 && !seen[e] && nl < 12) { seen[e] = true; loop[nl++] = e; e = next[e]; }
            for (int i = 1; i + 1 < nl && out + 3 <= 15; ++i) {
                T.tri[cse][out++] = loop[0];
                T.tri[cse][out++] = loop[i + 1];
                T.tri[cse][out++] = loop[i];
            }
        }
        T.num_vertices[cse] = (uint32_t)out;
        for (int k = out; k < 16; ++k) T.tri[cse][k] = -1;
    }
}

static McTables build_tables(const char*& origin) {
    McTables T;
#ifdef PMS_HAVE_REF_MC_TABLES
    for (int c = 0; c < 256; ++c) {
        T.edge_flags[c] = kRefEdgeFlags[c];
        T.num_vertices[c] = kRefNumVertices[c];
        for (int k = 0; k < 16; ++k) T.tri[c][k] = kRefTriangles[c][k];
    }
    for (int e = 0; e < 12; ++e) { T.edge_vertex[e][0] = kRefEdgeVertices[e][0]; T.edge_vertex[e][1] = kRefEdgeVertices[e][1]; }
    origin = "reference";
#else
    derive_tables(T);
    origin = "derived";
#endif
    return T;
}

static const char* g_origin = nullptr;

const McTables& mc_tables_host() {
    static const McTables T = build_tables(g_origin);
    return T;
}

const char* mc_tables_origin() {
    mc_tables_host();
    return g_origin;
}

// the derived tables, regardless of which set is active (for tests)
const McTables& mc_tables_derived() {
    static const McTables T = [] { McTables t; derive_tables(t); return t; }();
    return T;
}

}  // namespace pms

extern "C" {
// Copies the active tables (and whether they came from the reference tree).
// Exported for parity tests; not part of pms.h's stable surface.
int pms_mc_tables(uint32_t* edge_flags, int32_t* tri, uint32_t* num_vertices, uint32_t* edge_vertices, int derived) {
    const pms::McTables& T = derived ? pms::mc_tables_derived() : pms::mc_tables_host();
    if (edge_flags) memcpy(edge_flags, T.edge_flags, sizeof(T.edge_flags));
    if (tri) memcpy(tri, T.tri, sizeof(T.tri));
    if (num_vertices) memcpy(num_vertices, T.num_vertices, sizeof(T.num_vertices));
    if (edge_vertices) memcpy(edge_vertices, T.edge_vertex, sizeof(T.edge_vertex));
    return (!derived && strcmp(pms::mc_tables_origin(), "reference") == 0) ? 1 : 0;
}
}
