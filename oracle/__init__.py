"""The oracle: a CPU restatement of the reference's USL step plus build
recipes for the reference's own sources.  Test infrastructure only."""
