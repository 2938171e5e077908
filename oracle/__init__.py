"""CPU oracle for the ReaxFF evaluation path (test infrastructure, not product code).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package, and only as the checker or the timed CPU baseline.
The product path (``xreac_gb300``) never imports it.
"""

from .reaxff_oracle import COMPONENTS, evaluate, neighbor_list  # noqa: F401
