"""Workload definitions: flow past a z-aligned circular cylinder.

Grid sizes, domain lengths, Reynolds numbers and time steps of the five
cylinder-wake workloads this library is measured on, plus two small grids used
for golden vectors.  The cylinder has diameter 1 and sits at (5, ly/2); the
reference hard-codes the radius 0.5 and the centre height ly/2
(inc/dfib/setEta.hpp:145-147) and this module keeps both.

Boundary tables follow the reference's Dir/Num convention
(inc/BoundaryCondition/Boundary_Condition.hpp:4-31, 77-142): for face b and
component c the normal component gets ghost = Dir + Num*interior and a
tangential component gets ghost = 2 Dir + (2 Num - 1)*interior.  Faces are
0/1 = x-/x+, 2/3 = y-/y+, 4/5 = z-/z+; components 0/1/2 = u/v/w.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

# Uniform inflow u = 1 at x-, zero-gradient outflow at x+, free-slip walls in
# y (v = 0, du/dy = dw/dy = 0) and zero-gradient in z.  This is the closest
# table the reference can express to "inflow / outflow / free-slip / spanwise"
# (the reference has no periodic or convective-outflow option).
BC_CYLINDER_DIR = (
    (1.0, 0.0, 0.0),
    (0.0, 0.0, 0.0),
    (0.0, 0.0, 0.0),
    (0.0, 0.0, 0.0),
    (0.0, 0.0, 0.0),
    (0.0, 0.0, 0.0),
)
BC_CYLINDER_NUM = (
    (0.0, 0.0, 0.0),
    (1.0, 1.0, 1.0),
    (1.0, 0.0, 1.0),
    (1.0, 0.0, 1.0),
    (1.0, 1.0, 1.0),
    (1.0, 1.0, 1.0),
)


@dataclass(frozen=True)
class Workload:
    name: str
    nxc: int
    nyc: int
    nzc: int
    lx: float
    ly: float
    lz: float
    re: float
    dt: float
    steps: int
    tol: float = 1e-8
    omega: float = 1.7
    cx: float = 5.0
    cy: float | None = None  # None -> ly / 2 as in the reference
    radius: float = 0.5
    nsub: int = 100
    bc_dir: tuple = field(default=BC_CYLINDER_DIR)
    bc_num: tuple = field(default=BC_CYLINDER_NUM)

    @property
    def center_y(self) -> float:
        return self.ly / 2.0 if self.cy is None else self.cy

    @property
    def n_cells(self) -> int:
        return self.nxc * self.nyc * self.nzc

    @property
    def n_ghosted(self) -> int:
        return (self.nxc + 4) * (self.nyc + 4) * (self.nzc + 4)

    def with_(self, **kw) -> "Workload":
        return replace(self, **kw)


WORKLOADS = {
    # golden-vector grids (small enough to store full fields as fixtures)
    "g0": Workload("g0", 10, 8, 6, 2.5, 2.0, 0.75, re=100.0, dt=2e-3, steps=5, cx=1.0),
    "g1": Workload("g1", 16, 12, 6, 4.0, 3.0, 0.75, re=100.0, dt=2e-3, steps=10, cx=1.5),
    "g2": Workload("g2", 24, 20, 8, 6.0, 5.0, 1.0, re=100.0, dt=2e-3, steps=10, cx=2.0),
    # stretched-grid case: the reference's SML settings (fine region of 100
    # cells in x and y, offset -4 in x) need more than 100 interior cells
    "s1": Workload("s1", 120, 108, 8, 20.0, 10.0, 1.25, re=100.0, dt=1e-3, steps=10, cx=5.0),
    # profiling case: Krylov vectors (65 MB each) and per-kernel traffic above
    # the 129 MB L2, device footprint about 2 GB
    "p1": Workload("p1", 640, 320, 40, 20.0, 10.0, 1.25, re=100.0, dt=5e-4, steps=2, tol=1e-10),
    # the five cylinder-wake workloads
    "c1": Workload("c1", 128, 64, 8, 20.0, 10.0, 1.25, re=100.0, dt=2e-3, steps=200, tol=1e-8),
    "c2": Workload("c2", 512, 256, 32, 20.0, 10.0, 1.25, re=100.0, dt=5e-4, steps=2000, tol=1e-10),
    "c3": Workload("c3", 1024, 512, 64, 20.0, 10.0, 1.25, re=150.0, dt=5e-4, steps=1000, tol=1e-10),
    "c4": Workload("c4", 256, 128, 16, 20.0, 10.0, 1.25, re=100.0, dt=2e-3, steps=500, tol=1e-10),
    "c5": Workload("c5", 1536, 768, 96, 20.0, 10.0, 1.25, re=200.0, dt=5e-4, steps=400, tol=1e-10),
}
