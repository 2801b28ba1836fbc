"""Meshes of the voxelizer parity cases: closed triangle surfaces in lattice
units with the box they are voxelized in."""
from palabos_gb300 import meshes

CASES = {
    "sphere": (lambda: meshes.sphere((15.3, 16.7, 14.1), 9.2, 1280), (32, 34, 30)),
    "sphere_integer_centre": (lambda: meshes.sphere((16.0, 15.0, 17.0), 8.0, 320), (33, 31, 35)),
    "box_fractional": (lambda: meshes.cuboid((5.5, 6.25, 4.75), (20.5, 18.25, 22.75), (3, 2, 4)), (28, 26, 30)),
    "box_on_cell_centres": (lambda: meshes.cuboid((5, 6, 4), (20, 18, 22), (3, 2, 4)), (28, 26, 30)),
    "two_bodies": (lambda: meshes.merge(meshes.sphere((11.2, 15.3, 14.6), 6.1, 320),
                                        meshes.cuboid((23.31, 8.62, 9.41), (33.57, 21.38, 19.66))), (40, 30, 30)),
    "thin_box": (lambda: meshes.cuboid((3.37, 4.21, 5.62), (30.41, 5.83, 22.29), (5, 1, 3)), (34, 12, 28)),
}

# A thin box with half-integer faces: diagonal neighbour segments of the
# flood pass exactly through its edges.
EDGE_TOUCH = ((3.5, 4.25, 5.5), (30.5, 5.75, 22.5), (5, 1, 3), (34, 12, 28))

WIDTHS = (0, 1, 2)
