"""The reference's import name for this path: ``import snapy`` gives
snapy_gb300's drop-in surface (MeshBlockOptions.from_yaml, MeshBlock and the
index constants) as the reference's ``snapy`` module exposes them
(python/csrc/pymesh.cpp:19-381), so a caller's ``snapy.MeshBlock(...)``
runs on the GB300 path unchanged."""
from snapy_gb300 import *  # noqa: F401,F403
from snapy_gb300 import __all__, __version__  # noqa: F401
