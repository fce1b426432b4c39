/* libtiff is only used for input I/O; the oracle reads raw or Analyze. */
