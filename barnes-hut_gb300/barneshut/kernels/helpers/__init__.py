from .grid import next_perfect_square, get_bounding_box, get_neighbor_cells
from .grid import remove_bottom_left_neighbors
