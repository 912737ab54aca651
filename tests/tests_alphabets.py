"""Random-input alphabets of the reference's GPU/CPU cross-check
(bench/bench_boundary.cu:349-354)."""
ALPHABETS = {
    "json": b"{}[]:,\"\\0123456789tfn.-eE \n",
    "csv": b",.\n\r\"abc0123 ",
    "toml": b"[]{}.,=\"'#\nabc0123 \n",
    "clike": b"{};/*\n abc123",
    "ini": b"[]=;\n abc0123",
    "xml": b"<>/=?!\"' ab0123",
}
