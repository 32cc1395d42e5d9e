"""GB300-native VX3 step (vx3g): Python side of the C-ABI library.

The package directory name is not a Python identifier, so it is loaded under
the module name ``vx3g`` (see ``__graft_entry__.load_package``).
"""
