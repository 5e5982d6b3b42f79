// The reference's output files, written from the library's state:
//   finalResult_mesh.obj   TriMesh::saveAsMesh + TriMesh::save
//                          (src/TriMesh.cpp:1758-1969)
//   energyValPerIter.txt   Optimizer::writeEnergyValToFile (src/Optimizer.cpp:706-728)
//   gradientPerIter.txt    Optimizer::writeGradL2NormToFile (src/Optimizer.cpp:729-740)
//   info.txt               saveInfoForPresent (src/main.cpp:346-387) with
//                          TriMesh::computeStandardStretch (src/TriMesh.cpp:1585-1651)
// Numbers are printed as a default-formatted std::ostream prints them (six
// significant digits; the OBJ coordinates in scientific notation), so the
// files read like the reference's.
#include "optcuts_gpu.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

namespace {

struct HostMesh {
    int nV = 0, nF = 0, nC = 0;
    std::vector<double> Vr, UV;
    std::vector<int> F, cohE;
};

int read_mesh(oc_mesh* m, HostMesh& h)
{
    int rc = oc_mesh_get_topology(m, &h.nV, &h.nF, &h.nC, nullptr, nullptr, nullptr);
    if (rc) return rc;
    h.Vr.resize(3 * (size_t)h.nV);
    h.UV.resize(2 * (size_t)h.nV);
    h.F.resize(3 * (size_t)h.nF);
    h.cohE.resize(4 * (size_t)h.nC);
    rc = oc_mesh_get_topology(m, nullptr, nullptr, nullptr, h.F.data(), h.Vr.data(), h.cohE.data());
    if (rc) return rc;
    return oc_mesh_get_uv(m, h.UV.data());
}

int find_root(std::vector<int>& p, int a)
{
    while (p[a] != a) a = p[a] = p[p[a]];
    return a;
}

// TriMesh::computeStandardStretch: per triangle the deformation gradient
// from the rest triangle laid flat to its UV triangle, the L2 and L-inf
// stretch, shear and compression, area-weighted, scaled by the UV/rest
// area ratio
void standard_stretch(const HostMesh& h, double out[4])
{
    double l2 = 0.0, linf = -DBL_MAX, shear = 0.0, cinf = DBL_MAX, area = 0.0, areaUV = 0.0;
    for (int t = 0; t < h.nF; ++t) {
        const double* p[3];
        const double* u[3];
        for (int k = 0; k < 3; ++k) {
            p[k] = &h.Vr[3 * (size_t)h.F[3 * t + k]];
            u[k] = &h.UV[2 * (size_t)h.F[3 * t + k]];
        }
        const double e0[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
        const double e1[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
        const double cx = e0[1] * e1[2] - e0[2] * e1[1], cy = e0[2] * e1[0] - e0[0] * e1[2],
                     cz = e0[0] * e1[1] - e0[1] * e1[0];
        const double x1 = std::sqrt(e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2]);
        const double x2x = (e0[0] * e1[0] + e0[1] * e1[1] + e0[2] * e1[2]) / x1;
        const double x2y = std::sqrt(cx * cx + cy * cy + cz * cz) / x1;
        const double triArea = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
        const double a0 = u[1][0] - u[0][0], a1 = u[1][1] - u[0][1];
        const double b0 = u[2][0] - u[0][0], b1 = u[2][1] - u[0][1];
        const double len = std::sqrt(a0 * a0 + a1 * a1);
        // U = [len, (a.b)/len; 0, (a x b)/len], V = [x1 x2x; 0 x2y], Fg = V U^-1
        const double U00 = len, U01 = (a0 * b0 + a1 * b1) / len, U11 = (a0 * b1 - a1 * b0) / len;
        const double det = U00 * U11;
        const double i00 = U11 / det, i01 = -U01 / det, i11 = U00 / det;
        const double f00 = x1 * i00, f01 = x1 * i01 + x2x * i11, f10 = 0.0, f11 = x2y * i11;
        const double a = f00 * f00 + f10 * f10, b = f00 * f01 + f10 * f11, c = f01 * f01 + f11 * f11;
        const double t0 = a + c, t1 = std::sqrt((a - c) * (a - c) + 4.0 * b * b);
        const double tau = std::sqrt((t0 + t1) / 2.0), gamma = std::sqrt((t0 - t1) / 2.0);
        l2 += t0 / 2.0 * triArea;
        linf = std::max(linf, tau);
        shear += b * b / a / c * triArea;
        cinf = std::min(cinf, gamma);
        area += triArea;
        areaUV += 0.5 * (a0 * b1 - a1 * b0);
    }
    const double s = std::sqrt(areaUV / area);
    out[0] = std::sqrt(l2 / area) * s;
    out[1] = linf * s;
    out[2] = std::sqrt(shear / area);
    out[3] = cinf * s;
}

// Eigen's default matrix printing: columns right-aligned to their widest entry
std::string matrix_text(const std::vector<int>& M, int cols)
{
    const size_t rows = cols ? M.size() / cols : 0;
    std::vector<size_t> w(cols, 0);
    for (size_t r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) w[c] = std::max(w[c], std::to_string(M[r * cols + c]).size());
    std::ostringstream o;
    for (size_t r = 0; r < rows; ++r) {
        for (int c = 0; c < cols; ++c) {
            if (c) o << ' ';
            o << std::setw((int)w[c]) << M[r * cols + c];
        }
        if (r + 1 < rows) o << '\n';
    }
    return o.str();
}

} // namespace

extern "C" {

int oc_mesh_write_obj(oc_mesh* m, const char* path, const int* F0, int nV0, int scaleUV)
{
    if (!m || !path) return OC_ERR_INVALID;
    HostMesh h;
    int rc = read_mesh(m, h);
    if (rc) return rc;
    std::vector<double> V3, UVo(h.UV);
    std::vector<int> Fv(3 * (size_t)h.nF), Ft(h.F);
    if (F0) {   // saveAsMesh(path, F0): the input mesh's vertex numbering
        if (nV0 <= 0) return OC_ERR_INVALID;
        for (long long i = 0; i < 3LL * h.nF; ++i)
            if (F0[i] < 0 || F0[i] >= nV0) return OC_ERR_INVALID;
        V3.assign(3 * (size_t)nV0, 0.0);
        for (int t = 0; t < h.nF; ++t)
            for (int k = 0; k < 3; ++k)
                for (int d = 0; d < 3; ++d)
                    V3[3 * (size_t)F0[3 * t + k] + d] = h.Vr[3 * (size_t)h.F[3 * t + k] + d];
        std::copy(F0, F0 + 3 * (size_t)h.nF, Fv.begin());
    }
    else {   // saveAsMesh(path): copies glued back along the interior cohesive edges
        std::vector<int> par(h.nV);
        std::iota(par.begin(), par.end(), 0);
        for (int c = 0; c < h.nC; ++c) {
            const int* e = &h.cohE[4 * (size_t)c];
            if (std::min(std::min(e[0], e[1]), std::min(e[2], e[3])) < 0) continue;
            for (int p = 0; p < 2; ++p) {
                const int a = find_root(par, e[p]), b = find_root(par, e[2 + p]);
                if (a != b) par[std::max(a, b)] = std::min(a, b);
            }
        }
        std::vector<int> id(h.nV, -1);
        int n = 0;
        for (int v = 0; v < h.nV; ++v)
            if (find_root(par, v) == v) id[v] = n++;
        V3.assign(3 * (size_t)n, 0.0);
        std::vector<int> cnt(n, 0);
        for (int v = 0; v < h.nV; ++v) {
            const int g = id[find_root(par, v)];
            for (int d = 0; d < 3; ++d) V3[3 * (size_t)g + d] += h.Vr[3 * (size_t)v + d];
            ++cnt[g];
        }
        for (int g = 0; g < n; ++g)
            for (int d = 0; d < 3; ++d) V3[3 * (size_t)g + d] /= cnt[g];
        for (size_t i = 0; i < Fv.size(); ++i) Fv[i] = id[find_root(par, h.F[i])];
    }
    if (scaleUV && h.nV) {
        double lo[2] = {DBL_MAX, DBL_MAX}, hi[2] = {-DBL_MAX, -DBL_MAX};
        for (int v = 0; v < h.nV; ++v)
            for (int d = 0; d < 2; ++d) {
                lo[d] = std::min(lo[d], UVo[2 * (size_t)v + d]);
                hi[d] = std::max(hi[d], UVo[2 * (size_t)v + d]);
            }
        const double sc = std::max(hi[0] - lo[0], hi[1] - lo[1]);
        for (int v = 0; v < h.nV; ++v)
            for (int d = 0; d < 2; ++d) UVo[2 * (size_t)v + d] = (UVo[2 * (size_t)v + d] - lo[d]) / sc;
    }
    std::ofstream out(path);
    if (!out) return OC_ERR_INVALID;
    out << std::scientific;
    for (size_t v = 0; v < V3.size() / 3; ++v)
        out << "v " << V3[3 * v] << " " << V3[3 * v + 1] << " " << V3[3 * v + 2] << "\n";
    for (int v = 0; v < h.nV; ++v) out << "vt " << UVo[2 * (size_t)v] << " " << UVo[2 * (size_t)v + 1] << "\n";
    for (int t = 0; t < h.nF; ++t)
        out << "f " << Fv[3 * t] + 1 << "/" << Ft[3 * t] + 1 << " " << Fv[3 * t + 1] + 1 << "/" << Ft[3 * t + 1] + 1
            << " " << Fv[3 * t + 2] + 1 << "/" << Ft[3 * t + 2] + 1 << "\n";
    return out ? OC_OK : OC_ERR_INVALID;
}

int oc_optcuts_write(oc_optcuts* oc, const char* dir, const int* F0, int nV0, double lambdaInit)
{
    if (!oc || !dir) return OC_ERR_INVALID;
    const std::string d = std::string(dir) + (dir[0] && dir[std::string(dir).size() - 1] != '/' ? "/" : "");
    int n = 0;
    int rc = oc_optcuts_trace(oc, &n, nullptr);
    if (rc) return rc;
    std::vector<double> tr(7 * (size_t)n);
    rc = oc_optcuts_trace(oc, &n, tr.data());
    if (rc) return rc;
    {
        std::ofstream e(d + "energyValPerIter.txt"), g(d + "gradientPerIter.txt");
        if (!e || !g) return OC_ERR_INVALID;
        for (int i = 0; i < n; ++i) {
            const double* r = &tr[7 * (size_t)i];
            const double param = 1.0 - r[4];
            e << r[1] << " " << r[2] << " " << r[3] << " " << param << "\n";
            g << r[6] << " " << r[6] / (param * param) << "\n";
        }
    }
    double st[12];
    rc = oc_optcuts_state(oc, st);
    if (rc) return rc;
    oc_mesh* mesh = nullptr;
    rc = oc_optcuts_mesh(oc, &mesh);
    if (rc) return rc;
    HostMesh h;
    rc = read_mesh(mesh, h);
    if (rc) return rc;
    int nInit = 0;
    rc = oc_optcuts_initial_seams(oc, &nInit, nullptr);
    if (rc) return rc;
    std::vector<int> seams(4 * (size_t)nInit);
    rc = oc_optcuts_initial_seams(oc, &nInit, seams.data());
    if (rc) return rc;
    double stretch[4];
    standard_stretch(h, stretch);
    std::ofstream info(d + "info.txt");
    if (!info) return OC_ERR_INVALID;
    const double totalS = st[11] / 1000.0, newtonS = st[8] / 1000.0, topoS = (st[9] + st[10]) / 1000.0,
                 applyS = st[10] / 1000.0;
    info << (nV0 > 0 ? nV0 : h.nV) << " " << h.nF << "\n";
    info << (int)st[4] << " " << (int)st[5] << " 0 0 " << lambdaInit << " " << st[2] << "\n";
    info << "0.0 0.0 " << totalS << " " << totalS << " topo" << topoS << " desc" << newtonS << " scaf0 enUp" << applyS
         << " mtrComp0 mtrAssem0 symFac0 numFac0 backSolve0 lineSearch0 bSplit0 iSplit0 cMerge0\n";
    info << st[0] << " " << st[1] << "\n";
    info << stretch[0] << " " << stretch[1] << " " << stretch[2] << " " << stretch[3] << "\n";
    info << "initialSeams " << nInit << "\n" << matrix_text(seams, 4) << "\n";
    if (!info) return OC_ERR_INVALID;
    return oc_mesh_write_obj(mesh, (d + "finalResult_mesh.obj").c_str(), F0, nV0, 0);
}

} // extern "C"
