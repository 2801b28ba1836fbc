// CPU check of the library's state codec (palabos_gb300/csrc/dynstate.h)
// against a lattice state with dynamic content that the reference wrote:
// every cell of every component is decoded with plbgpu_dyn::readCell, then
// re-encoded with plbgpu_dyn::appendCell under the state's own registry ids,
// followed by its static values; the result must be the data file byte for
// byte.  Needs no GPU.
//
//   dynstate_check <state.plb> <state.dat> <nx> <ny> <nz>
//
// Prints "ok <cells>" and exits 0, or prints the first difference and exits 1.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../palabos_gb300/csrc/dynstate.h"

namespace {

std::string slurp(const char* path) {
    std::ifstream f(path, std::ios::binary);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// Inner text of every <tag ...> ... </tag> element, in order.
std::vector<std::string> elements(const std::string& doc, const std::string& tag) {
    std::vector<std::string> out;
    size_t a = 0;
    while ((a = doc.find("<" + tag, a)) != std::string::npos) {
        const char after = doc[a + 1 + tag.size()];
        if (after != '>' && after != ' ') { ++a; continue; }
        const size_t open = doc.find('>', a), close = doc.find("</" + tag + ">", open);
        out.push_back(doc.substr(open + 1, close - open - 1));
        a = close;
    }
    return out;
}

std::vector<long long> numbers(const std::string& text) {
    std::vector<long long> v;
    std::istringstream is(text);
    long long x;
    while (is >> x) v.push_back(x);
    return v;
}

int die(const char* what) {
    std::printf("FAIL %s\n", what);
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 6) return die("usage: dynstate_check <plb> <dat> <nx> <ny> <nz>");
    const std::string plb = slurp(argv[1]), dat = slurp(argv[2]);
    const int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]), nz = std::atoi(argv[5]);
    const int w = (int)numbers(elements(plb, "cellDim").at(0)).at(0);
    const std::vector<long long> offsets = numbers(elements(plb, "Offsets").at(0));
    const std::vector<std::string> comps = elements(plb, "Component");
    // DynamicsDict: <name> id </name>
    std::map<int, std::string> names;
    std::map<std::string, int> ids;
    {
        const std::string dd = elements(plb, "DynamicsDict").at(0);
        size_t p = 0;
        while ((p = dd.find('<', p)) != std::string::npos) {
            const size_t gt = dd.find('>', p);
            const std::string name = dd.substr(p + 1, gt - p - 1);
            const size_t close = dd.find("</" + name + ">", gt);
            const int id = (int)numbers(dd.substr(gt + 1, close - gt - 1)).at(0);
            names[id] = name;
            ids[name] = id;
            p = close + name.size() + 3;
        }
    }
    std::vector<char> again;
    size_t pos = 0;
    long long cells = 0;
    for (size_t i = 0; i < comps.size(); ++i) {
        const std::vector<long long> b = numbers(comps[i]);
        for (long long x = b[0]; x <= b[1]; ++x)
            for (long long y = b[2]; y <= b[3]; ++y)
                for (long long z = b[4]; z <= b[5]; ++z) {
                    plbgpu_dyn::Cell c;
                    const std::string err =
                        plbgpu_dyn::readCell(dat.data(), dat.size(), pos, names, (int)x, (int)y, (int)z, nx, ny, nz, c);
                    if (!err.empty()) return die(err.c_str());
                    plbgpu_dyn::Params p;
                    p.omega = c.omega;
                    p.bbRho = c.rho;
                    if (c.hasInvRho0 && !plbgpu_dyn::rho0FromInverse(c.invRho0, p.rho0)) return die("rho0");
                    plbgpu_dyn::appendCell(again, c.kind, c.bc, c.mask, p, &ids);
                    again.insert(again.end(), dat.data() + pos, dat.data() + pos + w * sizeof(double));
                    pos += w * sizeof(double);
                    ++cells;
                }
        if ((long long)pos != offsets.at(i)) return die("component size");
    }
    if (pos != dat.size()) return die("trailing bytes");
    if (again.size() != dat.size() || std::memcmp(again.data(), dat.data(), dat.size()) != 0) {
        size_t k = 0;
        while (k < again.size() && k < dat.size() && again[k] == dat[k]) ++k;
        std::printf("FAIL re-encoded bytes differ from byte %zu (sizes %zu vs %zu)\n", k, again.size(), dat.size());
        return 1;
    }
    std::printf("ok %lld\n", cells);
    return 0;
}
