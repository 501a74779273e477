"""CPU oracle (test infrastructure only): a NumPy restatement of the reference
µSpectre Newton-CG path.  Imported only by tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``; never by the product package."""
from .muspectre_oracle import *  # noqa: F401,F403
