// COMSOL text-mesh reader (read_comsol_mesh, src/3d/read_comsol.jl:9-54) for
// callers that build the mesh descriptor on the C side.
//
// The file is scanned line by line; lines shorter than 4 characters are
// skipped; after the exact header lines "# Mesh vertex coordinates",
// "# Elements" and "# Geometric entity indices" every line up to the next empty
// line is one coordinate triple, one element (its node numbers, 0-based in the
// file) or one entity index.  Element node numbers become 1-based and 6-node
// triangles get their rows 5 and 6 swapped (COMSOL orders the edge nodes
// differently from the 6-node triangle of the library).
#include "bie_internal.h"

#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace bie {

namespace {

void rstrip_cr(std::string &s) {
    while (!s.empty() && (s.back() == '\r' || s.back() == '\n')) s.pop_back();
}

bool blank(const std::string &s) {
    for (char ch : s)
        if (ch != ' ' && ch != '\t') return false;
    return true;
}

}  // namespace

void read_comsol(const std::string &path_in, std::vector<double> &coords, std::vector<int64_t> &topo, int &npe,
                 std::vector<int64_t> &entities) {
    std::string path = path_in;
    const std::string ext = ".mphtxt";
    if (path.size() < ext.size() || path.compare(path.size() - ext.size(), ext.size(), ext) != 0) path += ext;
    std::ifstream in(path);
    if (!in) fail(BIE_ERR_INVALID, "cannot open " + path);
    coords.clear();
    topo.clear();
    entities.clear();
    npe = 0;
    std::string line;
    int64_t lineno = 0;
    auto bad = [&](const std::string &what) {
        fail(BIE_ERR_INVALID, path + ":" + std::to_string(lineno) + ": " + what);
    };
    while (std::getline(in, line)) {
        ++lineno;
        rstrip_cr(line);
        if (line.size() < 4) continue;
        const int section = line == "# Mesh vertex coordinates" ? 1
                            : line == "# Elements"               ? 2
                            : line == "# Geometric entity indices" ? 3
                                                                   : 0;
        if (!section) continue;
        while (std::getline(in, line)) {
            ++lineno;
            rstrip_cr(line);
            if (line.empty() || blank(line)) break;
            std::istringstream ss(line);
            if (section == 1) {
                double v[3];
                std::string extra;
                if (!(ss >> v[0] >> v[1] >> v[2]) || (ss >> extra)) bad("expected three coordinates");
                coords.insert(coords.end(), v, v + 3);
            } else if (section == 2) {
                std::vector<int64_t> row;
                int64_t t;
                while (ss >> t) row.push_back(t);
                if (!ss.eof()) bad("non-integer node number");
                if (npe == 0) npe = (int)row.size();
                if ((int)row.size() != npe || (npe != 3 && npe != 6)) bad("elements must all have 3 or 6 nodes");
                for (int64_t &v : row) {
                    if (v < 0) bad("negative node number");
                    v += 1;
                }
                if (npe == 6) std::swap(row[4], row[5]);
                topo.insert(topo.end(), row.begin(), row.end());
            } else {
                int64_t e;
                if (!(ss >> e)) bad("expected an entity index");
                entities.push_back(e);
            }
        }
    }
    if (coords.empty() || topo.empty()) fail(BIE_ERR_INVALID, path + ": no vertex coordinates or no elements");
    const int64_t nc = (int64_t)coords.size() / 3;
    for (int64_t v : topo)
        if (v > nc) fail(BIE_ERR_INVALID, path + ": element node number beyond the vertex list");
}

}  // namespace bie
