"""GB300 launch wrappers with the reference's kernels.* module layout and names."""
