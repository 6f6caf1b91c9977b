// grid.cu -- the reference's stretched "SML" grid (grid::unit_SML and
// grid::init_nonuniform_SML, inc/grid/structureGrid.hpp:326-405, with the
// ghost extrapolation of grid::init_gC_dx, :506-559).  Host code: the grid is
// set-up data, built once and handed to cfd_set_metrics.
//
// Per axis with n ghosted nodes-1 (= interior + 4), interior count nCal, fine
// region of nS cells over length lS: coarse spacing d = (l - lS)/(nCal - nS),
// fine spacing dS = lS/nS; node gC is 0; the first (nCal - nS)/2 + offset
// cells are coarse, the next nS fine, the rest coarse.  nS = 0 gives l/nCal.
// The reference requires (n - nS) even; widths then come from the nodes:
// Dx[i] = X[i+1] - X[i], Dxs[i] = (X[i+2] - X[i])/2 on [gC, n - gC - 1),
// ghosts copied from the nearest computed value (the last interior Dxs too).
#include <cmath>
#include <string>
#include <vector>

#include "context.h"

using namespace cfd;

namespace {

int unit_sml(std::vector<double> &a, double lS, int nS, int off, double l, int n, const char *axis)
{
    const int nCal = n - 2 * GC;
    if (nS < 0 || nS > nCal) return fail(CFD_ERR_ARG, std::string("SML fine cells out of range on ") + axis);
    a.assign((size_t)n + 1, 0.0);
    a[GC] = 0.0;
    if (nS != 0) {
        if ((n - nS) % 2 != 0) return fail(CFD_ERR_ARG, std::string("SML needs (n - nSml) even on ") + axis);
        if (nS == nCal) return fail(CFD_ERR_ARG, std::string("SML needs coarse cells on ") + axis);
        const double dS = lS / nS, d = (l - lS) / (nCal - nS);
        int nl0 = (nCal - nS) / 2;
        int ns0 = nl0 + nS;
        const int nl1 = ns0 + nl0;
        nl0 += off;
        ns0 += off;
        if (nl0 <= 0 || ns0 > nl1) return fail(CFD_ERR_ARG, std::string("SML offset out of range on ") + axis);
        for (int i = 0; i < nl0; ++i) a[i + GC + 1] = a[i + GC] + d;
        for (int i = nl0; i < ns0; ++i) a[i + GC + 1] = a[i + GC] + dS;
        for (int i = ns0; i < nl1; ++i) a[i + GC + 1] = a[i + GC] + d;
    } else {
        for (int i = GC; i < n - GC; ++i) a[i + 1] = a[i] + l / nCal;
    }
    return CFD_OK;
}

// grid::init_gC_dx for one axis: ghost nodes, widths, ghost widths
void ghost_widths(std::vector<double> &X, std::vector<double> &D, std::vector<double> &Ds, int n)
{
    X[1] = 2 * X[2] - X[3];
    X[0] = 2 * X[1] - X[2];
    X[n - 1] = 2 * X[n - 2] - X[n - 3];
    X[n] = 2 * X[n - 1] - X[n - 2];
    D.assign(n, 0.0);
    Ds.assign(n, 0.0);
    for (int i = GC; i < n - GC - 1; ++i) Ds[i] = (X[i + 2] - X[i]) / 2.0;
    for (int i = GC; i < n - GC - 1; ++i) D[i] = X[i + 1] - X[i];
    D[0] = D[1] = D[2];
    Ds[0] = Ds[1] = Ds[2];
    D[n - 1] = D[n - 2] = D[n - 3] = X[n - 2] - X[n - 3];
    Ds[n - 1] = Ds[n - 2] = Ds[n - 3] = Ds[n - 4];
}

}  // namespace

extern "C" {

int cfd_sml_default(cfd_sml_config *cfg)
{
    if (!cfg) return fail(CFD_ERR_ARG, "null argument");
    // grid::init_nonuniform_SML (structureGrid.hpp:383-395)
    const double frac[3] = {0.3, 0.3, 0.5};
    const int nfine[3] = {100, 100, 0}, off[3] = {-4, 0, 0};
    for (int a = 0; a < 3; ++a) {
        cfg->fine_fraction[a] = frac[a];
        cfg->fine_cells[a] = nfine[a];
        cfg->offset[a] = off[a];
    }
    return CFD_OK;
}

int cfd_sml_metrics(int nxc, int nyc, int nzc, double lx, double ly, double lz, const cfd_sml_config *cfg,
                    double *X, double *Y, double *Z, double *Dx, double *Dy, double *Dz, double *Dxs, double *Dys,
                    double *Dzs)
{
    if (!cfg || !X || !Y || !Z || !Dx || !Dy || !Dz || !Dxs || !Dys || !Dzs) return fail(CFD_ERR_ARG, "null argument");
    if (nxc < 4 || nyc < 4 || nzc < 4) return fail(CFD_ERR_ARG, "every interior dimension must be at least 4");
    const int n[3] = {nxc + 2 * GC, nyc + 2 * GC, nzc + 2 * GC};
    const double len[3] = {lx, ly, lz};
    const char *names[3] = {"x", "y", "z"};
    double *nodes[3] = {X, Y, Z}, *w[3] = {Dx, Dy, Dz}, *ws[3] = {Dxs, Dys, Dzs};
    for (int a = 0; a < 3; ++a) {
        std::vector<double> node, D, Ds;
        CKS(unit_sml(node, cfg->fine_fraction[a] * len[a], cfg->fine_cells[a], cfg->offset[a], len[a], n[a],
                     names[a]));
        ghost_widths(node, D, Ds, n[a]);
        for (int i = 0; i <= n[a]; ++i) nodes[a][i] = node[i];
        for (int i = 0; i < n[a]; ++i) {
            w[a][i] = D[i];
            ws[a][i] = Ds[i];
        }
    }
    return CFD_OK;
}

int cfd_grid_sml(cfd_ctx *c, const cfd_sml_config *cfg)
{
    CKS(check_ctx(c));
    const Geo &g = c->g;
    std::vector<double> X(g.nx + 1), Y(g.ny + 1), Z(g.nz + 1), Dx(g.nx), Dy(g.ny), Dz(g.nz), Dxs(g.nx), Dys(g.ny),
        Dzs(g.nz);
    CKS(cfd_sml_metrics(g.nxc, g.nyc, g.nzc, c->cfg.lx, c->cfg.ly, c->cfg.lz, cfg, X.data(), Y.data(), Z.data(),
                        Dx.data(), Dy.data(), Dz.data(), Dxs.data(), Dys.data(), Dzs.data()));
    return cfd_set_metrics(c, X.data(), Y.data(), Z.data(), Dx.data(), Dy.data(), Dz.data(), Dxs.data(), Dys.data(),
                           Dzs.data());
}

}  // extern "C"
