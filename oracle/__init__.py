"""CPU parity oracle for the FastNoise2 node-tree path (test infrastructure only).

``tree``   -- node registry, tree model, encoded-tree codec (pure Python)
``oracle`` -- ctypes front-end to the C restatement in ``fn_oracle.c``

Nothing in the product package imports this package.
"""
