"""CPU oracle for the rubix particle -> IFU datacube path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` (``cpu_baseline`` and ``--impl reference``) may import this
package, and only as the checker or as the timed CPU baseline.  The product package
``rubix_gb300`` never imports it.
"""

from .ifu_oracle import *  # noqa: F401,F403
