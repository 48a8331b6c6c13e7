"""``cupyx.scipy`` stand-in: the SciPy modules the reference imports."""
import scipy.linalg as linalg  # noqa: F401
import scipy.ndimage as ndimage  # noqa: F401
import scipy.sparse as sparse  # noqa: F401
