from .bcs import set_bc_x, set_bc_z  # noqa: F401
from .directions import Directions  # noqa: F401
from .initial import init  # noqa: F401
