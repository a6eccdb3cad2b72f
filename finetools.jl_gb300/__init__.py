"""GB300 finite-element assembly for FinEtools.jl users.

A from-scratch GPU implementation of FinEtools' assembly hot path: the
FEMMBase bilinear/linear forms (bilform_diffusion, bilform_lin_elastic,
bilform_dot, innerproduct, linform_dot, distribloads) on H8, H20, T4, T10 and
Q4 elements, assembled into a CSR pattern that is built once on the device,
with a deterministic colour-ordered scatter.  The compute runs in hand-written
sm_103a CUDA kernels behind the C ABI of include/fegpu.h (libfegpu.so); this
package is the host-side mirror of the reference's Julia interface.
"""
from ._native import FegpuError, load as load_library
from .batch import AssemblyBatch
from .serve import AssemblyServer, estimate_mesh_bytes
from .assembly import (DeviceMatrix, SysmatAssemblerGPU, SysmatAssemblerSparseDiagGPU,
                       SysmatAssemblerFFBlockGPU, SysmatAssemblerSparseHRZLumpingSymmGPU,
                       SysvecAssemblerFBlockGPU, SysvecAssemblerGPU, assemble,
                       conjugategradient, makematrix, makevector, matrix_blocked_dd,
                       matrix_blocked_df, matrix_blocked_fd, matrix_blocked_ff, startassembly,
                       vector_blocked_d, vector_blocked_f)
from .femm import (CSys, DataCache, DeforModelRed3D, ElementwiseData, FEMMBase, ForceIntensity,
                   IntegDomain, IsotropicElementwise, bilform_convection, bilform_diffusion, bilform_div_grad,
                   bilform_dot, bilform_masslike,
                   bilform_lin_elastic, connectionmatrix, distribloads, innerproduct,
                   linform_dot)
from .fesets import FESetH8, FESetH20, FESetQ4, FESetT4, FESetT10
from .fields import DOF_KIND_DATA, DOF_KIND_FREE, NodalField, gathersysvec, numberdofs, setebc
from .meshes import (FENodeSet, H8block, H8blockx, H8toH20, H20block, Q4block, Q4blockx,
                     T4block, T4blockx, T4toT10, T10block, h8_diffusion_mesh,
                     h20_elastic_mesh, isotropic_D, lame, linearspace, nearest_block,
                     t10_elastic_mesh)
from .rules import GaussRule, TetRule

__all__ = [n for n in dir() if not n.startswith("_")]
