/* empty: no LINPACK routine is used by the hot-path files */
