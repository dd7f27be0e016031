from .grid import next_perfect_square, get_bounding_box
