"""Algorithmic bytes of one time step, frozen from the device layout of the FP64 and FP32C paths.

Each persistent field a pass touches is counted once read and once written; each gather of a
voxel field by the link pass is counted once per voxel (not per link end); material tables are not
counted.  These are the figures bench.py divides by the CUDA-event time of each pass.

FP64 layout (voxelyze_gb300/csrc/vx_phys64.cuh):
  link pass, per link : endpoint ids 8, flags 4+4, material id 4, previous pos2/angle1v/angle2v 72
                        read + 72 written, rest length 8, transverse area/strain sum 8, strain /
                        maxStrain / strainOffset 12 read + strain/maxStrain/strainOffset/stress 16
                        written, forces and moments 96 written                          = 304 B
            per voxel : position 24, orientation 32, previous dt 4, material id 4      =  64 B
  Poisson pre-pass (nu != 0), per voxel: flags 4+4, 6 link ids 24, cached strain 12   =  44 B
                        (the link strains it gathers are counted once per link: 8 B)
  voxel pass, per voxel: pose and momenta 104 read + 104 written, flags 4+4, material id 4,
                        external id 4, 6 link ids 24, lattice index 12, temperature 4,
                        previous dt 4 written                                          = 268 B
            per link  : the force and moment each end gathers, 2 x 48                 =  96 B
"""
from __future__ import annotations

FP64_LINK_PER_LINK = 304
FP64_LINK_PER_VOXEL = 64
FP64_POISSON_PER_VOXEL = 44
FP64_POISSON_PER_LINK = 8
FP64_VOXEL_PER_VOXEL = 268
FP64_VOXEL_PER_LINK = 96


def fp64_bytes(n_voxels: int, n_links: int, poisson: bool) -> dict:
    link = FP64_LINK_PER_LINK * n_links + FP64_LINK_PER_VOXEL * n_voxels
    if poisson:
        link += FP64_POISSON_PER_VOXEL * n_voxels + FP64_POISSON_PER_LINK * n_links
    voxel = FP64_VOXEL_PER_VOXEL * n_voxels + FP64_VOXEL_PER_LINK * n_links
    return {"link": link, "voxel": voxel, "step": link + voxel}


# FP32C layout (voxelyze_gb300/csrc/vx_phys32.cuh):
#   link pass, per link : endpoint ids 8, flags 4 read, material id 4, previous pos2/angle2v 24 read
#                         + 24 written, rest offset 4, transverse area/strain sum 8 (written where
#                         the link material has nu != 0, read where nu == 0), maxStrain/strainOffset
#                         8 read, strain and stress 8 written, forces and moments 48 written = 144 B
#                         + previous angle1v 12 read + 12 written per large-angle link (a small-
#                         angle link's is zero: neither read nor rewritten while it stays small)
#                         (flags, maxStrain and strainOffset are written only when they change,
#                         which is rare, so those writes are not counted)
#             per voxel : displacement 12, orientation 16, material id 4                  =  32 B
#                         (+ the cached Poisson strain 12 when nu != 0)
#   voxel pass, per voxel: displacement and orientation with their compensations, momenta 80 read
#                         + 80 written, flags 4 read (written only when they change), material id
#                         4, external id 4, 6 link ids 24, lattice z 4, temperature 4     = 204 B
#             per link  : the force and moment each end gathers, 2 x 24                   =  48 B
#   Poisson cache (nu != 0), filled by the voxel pass for the next step: cached strain 12 B written
#                         per voxel, strain and strain ratio 8 B per link gathered
FP32C_LINK_PER_LINK = 144
FP32C_LINK_PER_LARGE_ANGLE_LINK = 24
FP32C_LINK_PER_VOXEL = 32
FP32C_LINK_PER_VOXEL_POISSON = 12
FP32C_VOXEL_PER_VOXEL = 204
FP32C_VOXEL_PER_LINK = 48
FP32C_VOXEL_PER_VOXEL_POISSON = 12
FP32C_VOXEL_PER_LINK_POISSON = 8


def fp32c_bytes(n_voxels: int, n_links: int, poisson: bool, large_angle_links: int = 0) -> dict:
    link = (FP32C_LINK_PER_LINK * n_links + FP32C_LINK_PER_LARGE_ANGLE_LINK * large_angle_links
            + FP32C_LINK_PER_VOXEL * n_voxels)
    voxel = FP32C_VOXEL_PER_VOXEL * n_voxels + FP32C_VOXEL_PER_LINK * n_links
    if poisson:
        link += FP32C_LINK_PER_VOXEL_POISSON * n_voxels
        voxel += FP32C_VOXEL_PER_VOXEL_POISSON * n_voxels + FP32C_VOXEL_PER_LINK_POISSON * n_links
    return {"link": link, "voxel": voxel, "step": link + voxel}


# DRAM bytes per launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum) on the
# 128x128x64 lattice, FP32C, warm step (profiles/fp32c_lattice128x128x64_dram.md), per unit
MEASURED_TRAFFIC = {
    "fp32c_link": {"per_voxel": 0.0, "per_link": 134.5},    # k_link32
    "fp32c_voxel": {"per_voxel": 332.3, "per_link": 0.0},   # k_voxel32 with the Poisson fill
}


def measured_traffic(kind: str, n_voxels: int, n_links: int):
    t = MEASURED_TRAFFIC.get(kind)
    if t is None:
        return None
    return t["per_voxel"] * n_voxels + t["per_link"] * n_links


# FP64 path against the FP64 pipe.  Double-precision instructions per unit counted by ncu
# (sm__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum and sm__inst_executed_pipe_fp64.sum)
# on a warm launch of each pass of the FP64 path on the bench's lattice generator at 48x48x24
# (46,964 voxels, 116,312 links), divided by the units of the launch
# (profiles/fp64_k_link_k_voxel_lattice48x48x24_counts.md).  The DFMAs are the iterations of IEEE
# division and square root (the FP64 path is compiled without contraction); their count varies by
# ~20 % between steps with the operands.  FLOPs count an FMA as two.
FP64_OPS = {
    "link": {"dadd": 136.65, "dmul": 142.01, "dfma": 21.06, "pipe_warp_inst": 11.594},
    "voxel": {"dadd": 104.09, "dmul": 115.04, "dfma": 14.42, "pipe_warp_inst": 8.298},
}


def fp64_ops(n_voxels: int, n_links: int, poisson: bool):
    """FLOPs and FP64-pipe warp instructions of one FP64 link pass (and voxel pass) at this size, or
    None if the counts have not been measured."""
    L, V = FP64_OPS["link"], FP64_OPS["voxel"]
    if L is None:
        return None
    out = {"link_flops": (L["dadd"] + L["dmul"] + 2 * L["dfma"]) * n_links,
           "link_pipe_inst": L["pipe_warp_inst"] * n_links}
    if V is not None:
        out["voxel_flops"] = (V["dadd"] + V["dmul"] + 2 * V["dfma"]) * n_voxels
        out["voxel_pipe_inst"] = V["pipe_warp_inst"] * n_voxels
    return out
