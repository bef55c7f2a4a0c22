"""The benchmark workloads: seeded synthetic particle sets and the physics
each is run with (shared by bench.py and the autotuner).

c1  Plummer sphere a=1, N=16,384
c2  exponential disk (R_d=1, z_d=0.1, 80% of the mass) + Hernquist bulge, N=524,288
c3  two Plummer spheres a=1, M=0.5 each, separation 10, N=4,194,304
c4  256 Plummer systems, N_s log-uniform in [1024, 65536] (batched)
c5  uniform unit cube, log-normal masses, N=16,777,216, quoted at the
    reference's 7 layers (lbits 6) and at all 21 bits (lbits 21)
ref the reference's own scene (Renderer.swift:25-46,441-493): 5 stars and 200
    planets in the tree, 500,000 dust tracers, REFERENCE preset

Every set comes from the Philox4x32-10 generators of libastro_cuda
(astro_gb300.ic), keyed by the workload's seed, so the host and the GPU
see identical inputs.
"""
from __future__ import annotations

from dataclasses import dataclass, field


@dataclass(frozen=True)
class Workload:
    name: str
    description: str
    generator: str        # astro_gb300.ic function ("batch" = plummer_batch)
    n: int                # particles (0: set by the batch generator)
    seed: int
    dt: float
    physics: dict = field(default_factory=dict)   # astro_params overrides (softening, ...)
    lbits: int = 14       # tree depth the autotuner starts from
    preset: str = "physical"
    quoted_lbits: int | None = None  # tree depth the workload is quoted at (held fixed)

    def make_colors(self):
        """ColorType[] and the tree count of the REFERENCE scene."""
        from . import ic

        _, _, ct = ic.reference_scene(5, 200, self.n - 205, seed=self.seed)
        return ct, 205

    def make(self):
        """(PositionMass[], VelocityRadius[], system sizes or None)."""
        from . import ic

        if self.generator == "reference_scene":
            pm, vr, _ = ic.reference_scene(5, 200, self.n - 205, seed=self.seed)
            return pm, vr, None
        if self.generator == "batch":
            pm, vr, sizes = ic.plummer_batch(256, self.seed)
            return pm, vr, [int(s) for s in sizes]
        pm, vr = getattr(ic, self.generator)(self.n, self.seed)
        return pm, vr, None


WORKLOADS = {
    "c1": Workload("c1", "Plummer sphere a=1 N=16384", "plummer", 16384, 1001, 1e-3,
                   dict(softening=0.01)),
    "c2": Workload("c2", "exponential disk + Hernquist bulge N=524288", "disk_bulge", 524288,
                   1002, 5e-4, dict(softening=0.005)),
    "c3": Workload("c3", "two Plummer spheres a=1 M=0.5 at separation 10, N=4194304",
                   "two_plummer", 4194304, 1003, 1e-3, dict(softening=0.002)),
    "c4": Workload("c4", "256 Plummer systems, N_s log-uniform [1024, 65536]", "batch", 0, 1004,
                   1e-3, dict(softening=0.01)),
    "c5": Workload("c5", "uniform unit cube, log-normal masses, N=16777216", "uniform_cube",
                   16777216, 1005, 1e-3, dict(softening=0.001), quoted_lbits=6),
    "ref": Workload("ref", "the reference's scene: 5 stars + 200 planets in the tree, 500,000 dust "
                    "tracers (REFERENCE preset)", "reference_scene", 500205, 1, 1.0 / 60.0, {}, 6,
                    "reference"),
}
