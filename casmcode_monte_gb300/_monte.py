"""The core module's names under the path the reference binds them at
(``libcasm.monte._monte``, python/src/monte.cpp:106-109,385-553): the engine and
generator, the method log, ValueMap and its four typed maps."""
from . import (BooleanValueMap, MatrixValueMap, MethodLog, RandomNumberEngine,  # noqa: F401
               RandomNumberGenerator, ScalarValueMap, ValueMap, VectorValueMap, __version__)
