from .timing import TimedCodeBlock  # noqa: F401
from .utils import sample_ellipse_cosine  # noqa: F401
