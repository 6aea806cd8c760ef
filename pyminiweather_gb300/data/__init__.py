from .constants import Constants  # noqa: F401
from .fields import Fields, initialize_fields  # noqa: F401
from .quadrature import Quadrature  # noqa: F401
