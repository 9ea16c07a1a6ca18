"""tensormesh_gb300: GB300-native (sm_103a) tensorized FEM assembly.

A drop-in for the assembly path of TensorMesh: ``ElementAssembler`` /
``NodeAssembler`` and the built-in forms keep the reference's call
signatures and return types, and run hand-written CUDA kernels through the
C ABI of ``libtmgb300.so`` (``include/tensormesh_gb300.h``).
"""
from .mesh import Mesh, gen_unit_square, gen_unit_square_mixed, gen_unit_cube
from .element import element_type2dimension, element_type2order
from .transformation import Transformation, ReduceProjector, SparseProjector
from .sparse import SparseMatrix
from .assemble import ElementAssembler, NodeAssembler, assemble_forms
from .builtin import (LaplaceElementAssembler, DiffusionElementAssembler, MassElementAssembler,
                      LinearElasticityElementAssembler, const_node_assembler, func_node_assembler,
                      LoadNodeAssembler)
from .facet import FacetAssembler, LoadFacetAssembler, const_facet_assembler, func_facet_assembler
from .solve import bicgstab_solve, pcg_solve
from .condense import Condenser
from .adjoint import solve_diffusion
from . import autotune

__version__ = "0.1.0"

__all__ = [
    "Mesh", "gen_unit_square", "gen_unit_square_mixed", "gen_unit_cube", "Transformation", "ReduceProjector", "SparseProjector",
    "SparseMatrix", "ElementAssembler", "NodeAssembler", "assemble_forms", "LaplaceElementAssembler",
    "DiffusionElementAssembler", "MassElementAssembler", "LinearElasticityElementAssembler",
    "const_node_assembler", "func_node_assembler", "LoadNodeAssembler", "pcg_solve", "bicgstab_solve",
    "element_type2dimension", "element_type2order", "Condenser", "solve_diffusion",
    "FacetAssembler", "LoadFacetAssembler", "const_facet_assembler", "func_facet_assembler",
]
