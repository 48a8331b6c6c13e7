"""``cupyx.scipy`` stand-in: the SciPy modules the reference imports, registered
under the ``cupyx.scipy.*`` names so that ``import cupyx.scipy.linalg`` works."""
import sys

import scipy.linalg as linalg  # noqa: F401
import scipy.ndimage as ndimage  # noqa: F401
import scipy.sparse as sparse  # noqa: F401

sys.modules[__name__ + ".linalg"] = linalg
sys.modules[__name__ + ".ndimage"] = ndimage
sys.modules[__name__ + ".sparse"] = sparse
