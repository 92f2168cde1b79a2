// dsc_reader.cu -- the reference's input decks and node normals as library
// calls (host code).
//
// A deck is input.bem plus the files it names (src/depSolver.c:98-252,
// src/depSolver-shift.c:120-140,205-217): NODES (count, file), ELEMS (count,
// type, file), MATERIALS (count, then "id sigma eps_r" lines), INTERFACES
// (count, then "id mat_a mat_b"), PROBLEM(S) (frequency, boundary-condition
// file), optionally REPOSITION (first moved node, displacement: the
// position-sweep decks of depSolver-sft), ANALYSIS (solver "gauss" or
// "gmres preCond nInit", analysis type, and for types 5-11 the force points
// with the sphere radius or the ellipsoid's semi-axes), INTERNALPOINTS
// (count, STD|VTK, file) and COLUMNS.  Text after "//" on a line is a
// comment, as the reference's comFilter strips it (src/preProcess.c:48-81).
// Node, element and point files hold one record per line led by an index
// the reader discards; the boundary-condition file has 2N records "index
// type values" with types written as integers or "C<k>" (type k + 5), and
// 1, 2 or 3 values by type (src/depSolver.c:219-237).
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/depsolver_cuda.h"
#include "dsc_internal.h"
#include "dsc_quad8.h"

namespace dsc {

struct BemDeck {
    int nen = 6;
    unsigned N = 0, E = 0, nMat = 0, nIf = 0;
    std::vector<double> nodes, mbc, mat;
    std::vector<unsigned> elems, bctype, ifaces;
    double freq = 0.0;
    int gmres = 0;
    unsigned preCond = 0, nInit = 0;
    int analysis = 0;
    unsigned pNodes = 0;
    double dr[3] = {0.0, 0.0, 0.0};
    bool reposition = false;
    std::vector<double> internal, fpoints;
    double axis[3] = {0.0, 0.0, 0.0};
};

// The whitespace-separated tokens of a file with "//" comments removed.
static int tokens(const std::string &path, std::vector<std::string> &out)
{
    std::ifstream in(path);
    if (!in) {
        set_error("cannot open %s", path.c_str());
        return kErrArg;
    }
    out.clear();
    std::string line;
    while (std::getline(in, line)) {
        const size_t c = line.find("//");
        if (c != std::string::npos) line.resize(c);
        std::istringstream ls(line);
        std::string t;
        while (ls >> t) out.push_back(t);
    }
    return kOk;
}

struct Cursor {
    const std::vector<std::string> &t;
    size_t i = 0;
    std::string file;
    bool bad = false;
    const std::string &next()
    {
        static const std::string empty;
        if (i >= t.size()) {
            bad = true;
            return empty;
        }
        return t[i++];
    }
    double num()
    {
        const std::string &s = next();
        char *end = nullptr;
        const double v = strtod(s.c_str(), &end);
        if (s.empty() || *end) bad = true;
        return v;
    }
    unsigned uint()
    {
        const double v = num();
        if (v < 0 || v != floor(v)) bad = true;
        return (unsigned)v;
    }
    std::string upper()
    {
        std::string s = next();
        for (char &c : s) c = (char)toupper((unsigned char)c);
        return s;
    }
};

static std::string join(const std::string &dir, const std::string &f)
{
    if (f.empty() || f[0] == '/' || dir.empty()) return f;
    return dir + "/" + f;
}

static int read_deck(const std::string &dir, BemDeck &d)
{
    std::vector<std::string> tk;
    DSC_TRY(tokens(join(dir, "input.bem"), tk));
    Cursor c{tk};
    c.next();  // NODES
    d.N = c.uint();
    const std::string node_file = c.next();
    c.next();  // ELEMS
    d.E = c.uint();
    std::string etype = c.next();
    for (char &ch : etype) ch = (char)tolower((unsigned char)ch);
    const std::string elem_file = c.next();
    // the reference's names (src/preProcess.c:110-146); its driver takes
    // tria3 and tria6 (src/depSolver.c:180-183), this library also quad8
    if (etype.compare(0, 5, "tria6") == 0) d.nen = 6;
    else if (etype.compare(0, 5, "tria3") == 0) d.nen = 3;
    else if (etype.compare(0, 5, "quad8") == 0) d.nen = 8;
    else {
        set_error("element type %s: the path handles tria3, tria6 and quad8", etype.c_str());
        return kErrArg;
    }
    c.next();  // MATERIALS
    d.nMat = c.uint();
    for (unsigned k = 0; k < d.nMat && !c.bad; k++) {
        c.next();
        d.mat.push_back(c.num());
        d.mat.push_back(c.num());
    }
    c.next();  // INTERFACES
    d.nIf = c.uint();
    for (unsigned k = 0; k < d.nIf && !c.bad; k++) {
        c.next();
        d.ifaces.push_back(c.uint());
        d.ifaces.push_back(c.uint());
    }
    c.next();  // PROBLEM(S)
    d.freq = c.num();
    const std::string bc_file = c.next();
    std::string sec = c.upper();
    if (sec.compare(0, 10, "REPOSITION") == 0) {
        d.reposition = true;
        d.pNodes = c.uint();
        for (int k = 0; k < 3; k++) d.dr[k] = c.num();
        sec = c.upper();
    }
    // ANALYSIS
    const std::string solver = c.upper();
    if (solver == "GMRES") {
        d.gmres = 1;
        d.preCond = c.uint();
        d.nInit = c.uint();
    }
    d.analysis = (int)c.uint();
    std::string fpoint_file;
    unsigned nfp = 0;
    if (d.analysis > 4 && d.analysis < 10) {
        nfp = c.uint();
        d.axis[0] = c.num();
        fpoint_file = c.next();
    } else if (d.analysis == 10 || d.analysis == 11) {
        nfp = c.uint();
        for (int k = 0; k < 3; k++) d.axis[k] = c.num();
        fpoint_file = c.next();
    }
    c.next();  // INTERNALPOINTS
    const unsigned nint = c.uint();
    std::string out_type, int_file;
    if (nint > 0) {
        out_type = c.upper();
        int_file = c.next();
    }
    if (c.bad) {
        set_error("%s/input.bem: missing or malformed entries", dir.c_str());
        return kErrArg;
    }
    // nodes (shifted from pNodes on, as depSolver-sft does)
    DSC_TRY(tokens(join(dir, node_file), tk));
    {
        Cursor n{tk};
        d.nodes.resize(3 * (size_t)d.N);
        for (unsigned i = 0; i < d.N; i++) {
            n.next();
            for (int k = 0; k < 3; k++) d.nodes[3 * (size_t)i + k] = n.num();
        }
        if (n.bad) {
            set_error("%s: fewer than %u nodes", node_file.c_str(), d.N);
            return kErrArg;
        }
        if (d.reposition)
            for (unsigned i = d.pNodes; i < d.N; i++)
                for (int k = 0; k < 3; k++) d.nodes[3 * (size_t)i + k] += d.dr[k];
    }
    DSC_TRY(tokens(join(dir, elem_file), tk));
    {
        Cursor e{tk};
        d.elems.resize((size_t)d.nen * d.E);
        for (unsigned i = 0; i < d.E; i++) {
            e.next();
            for (int k = 0; k < d.nen; k++) d.elems[(size_t)d.nen * i + k] = e.uint();
        }
        if (e.bad) {
            set_error("%s: fewer than %u elements", elem_file.c_str(), d.E);
            return kErrArg;
        }
    }
    DSC_TRY(tokens(join(dir, bc_file), tk));
    {
        Cursor b{tk};
        d.bctype.resize(2 * (size_t)d.N);
        d.mbc.assign(6 * (size_t)d.N, 0.0);
        for (size_t j = 0; j < 2 * (size_t)d.N; j++) {
            b.next();
            const std::string s = b.next();
            unsigned t;
            if (!s.empty() && (s[0] == 'C' || s[0] == 'c')) t = (unsigned)atoi(s.c_str() + 1) + 5;
            else t = (unsigned)atoi(s.c_str());
            d.bctype[j] = t;
            const int nv = (t > 2 && t < 6) ? 3 : (t == 0 || t == 6) ? 2 : 1;
            for (int k = 0; k < nv; k++) d.mbc[3 * j + k] = b.num();
        }
        if (b.bad) {
            set_error("%s: fewer than %zu boundary conditions", bc_file.c_str(), 2 * (size_t)d.N);
            return kErrArg;
        }
    }
    if (nint > 0) {
        DSC_TRY(tokens(join(dir, int_file), tk));
        Cursor p{tk};
        if (out_type.compare(0, 3, "VTK") == 0)
            for (int k = 0; k < 6; k++) p.next();  // grid counts and spacings
        d.internal.resize(3 * (size_t)nint);
        for (unsigned i = 0; i < nint; i++) {
            p.next();
            for (int k = 0; k < 3; k++) d.internal[3 * (size_t)i + k] = p.num();
        }
        if (p.bad) {
            set_error("%s: fewer than %u points", int_file.c_str(), nint);
            return kErrArg;
        }
    }
    if (nfp > 0) {
        DSC_TRY(tokens(join(dir, fpoint_file), tk));
        Cursor p{tk};
        d.fpoints.resize(3 * (size_t)nfp);
        for (unsigned i = 0; i < nfp; i++) {
            p.next();
            for (int k = 0; k < 3; k++) d.fpoints[3 * (size_t)i + k] = p.num();
        }
        if (p.bad) {
            set_error("%s: fewer than %u force points", fpoint_file.c_str(), nfp);
            return kErrArg;
        }
    }
    return kOk;
}

}  // namespace dsc

using namespace dsc;

struct dsc_bem {
    BemDeck d;
};

extern "C" int dsc_bem_read(const char *dir, dsc_bem **out)
{
    *out = nullptr;
    if (!dir) {
        set_error("dsc_bem_read: no directory");
        return kErrArg;
    }
    dsc_bem *b = new dsc_bem();
    const int rc = read_deck(dir, b->d);
    if (rc != kOk) {
        delete b;
        return rc;
    }
    *out = b;
    return kOk;
}

extern "C" void dsc_bem_free(dsc_bem *b) { delete b; }

extern "C" int dsc_bem_info(const dsc_bem *b, int *nen, unsigned *N, unsigned *E, unsigned *nMat, unsigned *nIf,
                            double *freq, int *analysis, int *gmres, unsigned *preCond, unsigned *nInit,
                            unsigned *nInternal, unsigned *nForcePoints, int *reposition, unsigned *pNodes,
                            double *dr, double *axis)
{
    const BemDeck &d = b->d;
    if (nen) *nen = d.nen;
    if (N) *N = d.N;
    if (E) *E = d.E;
    if (nMat) *nMat = d.nMat;
    if (nIf) *nIf = d.nIf;
    if (freq) *freq = d.freq;
    if (analysis) *analysis = d.analysis;
    if (gmres) *gmres = d.gmres;
    if (preCond) *preCond = d.preCond;
    if (nInit) *nInit = d.nInit;
    if (nInternal) *nInternal = (unsigned)(d.internal.size() / 3);
    if (nForcePoints) *nForcePoints = (unsigned)(d.fpoints.size() / 3);
    if (reposition) *reposition = d.reposition ? 1 : 0;
    if (pNodes) *pNodes = d.pNodes;
    for (int k = 0; k < 3; k++) {
        if (dr) dr[k] = d.dr[k];
        if (axis) axis[k] = d.axis[k];
    }
    return kOk;
}

extern "C" int dsc_bem_arrays(const dsc_bem *b, double *nodes, unsigned *elems, unsigned *bctype, double *mbc,
                              double *mat, unsigned *ifaces, double *internal, double *force_points)
{
    const BemDeck &d = b->d;
    auto put = [](auto *dst, const auto &v) {
        if (dst) std::copy(v.begin(), v.end(), dst);
    };
    put(nodes, d.nodes);
    put(elems, d.elems);
    put(bctype, d.bctype);
    put(mbc, d.mbc);
    put(mat, d.mat);
    put(ifaces, d.ifaces);
    put(internal, d.internal);
    put(force_points, d.fpoints);
    return kOk;
}

extern "C" int dsc_node_normals(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                                double *normals)
{
    if ((nen != 3 && nen != 6 && nen != 8) || !nodes || !elems || !normals || N == 0) {
        set_error("dsc_node_normals: bad arguments");
        return kErrArg;
    }
    std::vector<int> e0((size_t)E * nen);
    for (size_t t = 0; t < e0.size(); t++) {
        if (elems[t] < 1 || elems[t] > N) {
            set_error("dsc_node_normals: element node id %u outside 1..%u", elems[t], N);
            return kErrArg;
        }
        e0[t] = (int)elems[t] - 1;
    }
    if (nen == 8) q8_node_normals((int)N, (int)E, nodes, e0.data(), normals);
    else node_normals(nen, (int)N, (int)E, nodes, e0.data(), normals);
    return kOk;
}
