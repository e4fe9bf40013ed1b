"""Comparators that bench.py times beside the product: the reference's own
ray traversal restated in CUDA (restated/).  Nothing here is on the product
path."""
