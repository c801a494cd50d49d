"""doma_gb300: GB300-native fixed-source discrete-ordinates sweep / source iteration."""
from . import abi, problems  # noqa: F401
