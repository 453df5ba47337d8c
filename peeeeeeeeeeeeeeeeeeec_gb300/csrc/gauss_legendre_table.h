/* Generated by gen_gauss_legendre.py; do not edit. */
#ifndef PEEC_GB300_GAUSS_LEGENDRE_TABLE_H
#define PEEC_GB300_GAUSS_LEGENDRE_TABLE_H
/* Row r holds order GL_ORDERS[r]; unused slots are 0. */
#define GL_NUM_ORDERS 9
static const int GL_ORDERS[GL_NUM_ORDERS] = {2, 3, 4, 5, 6, 8, 10, 12, 16};
static const double GL_NODES[GL_NUM_ORDERS][16] = {
    {-0x1.279a74590331cp-1, 0x1.279a74590331cp-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.8c97ef43f7248p-1, 0.0, 0x1.8c97ef43f7248p-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.b8e6dbcf63985p-1, -0x1.5c23fd9dd3dfcp-2, 0x1.5c23fd9dd3dfcp-2, 0x1.b8e6dbcf63985p-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.cff6ce0533a69p-1, -0x1.13b23fd99b705p-1, 0.0, 0x1.13b23fd99b705p-1, 0x1.cff6ce0533a69p-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.dd6ca4e80a01ep-1, -0x1.528a09655c95ep-1, -0x1.e8b12d03675c5p-3, 0x1.e8b12d03675c5p-3, 0x1.528a09655c95ep-1, 0x1.dd6ca4e80a01ep-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.ebab1cb0acc67p-1, -0x1.97e4ab249f41ep-1, -0x1.0d129583284b4p-1, -0x1.77ac94f3c7345p-3, 0x1.77ac94f3c7345p-3, 0x1.0d129583284b4p-1, 0x1.97e4ab249f41ep-1, 0x1.ebab1cb0acc67p-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.f2a3e062af2d8p-1, -0x1.bae995e9cb2f3p-1, -0x1.5bdb9228de198p-1, -0x1.bbcc009016adcp-2, -0x1.30e507891e27ap-3, 0x1.30e507891e27ap-3, 0x1.bbcc009016adcp-2, 0x1.5bdb9228de198p-1, 0x1.bae995e9cb2f3p-1, 0x1.f2a3e062af2d8p-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.f68f1d8e42e81p-1, -0x1.cee874ffb88b4p-1, -0x1.8a30aeed88f36p-1, -0x1.2cb4f05c077f9p-1, -0x1.78a8d20a8b19dp-2, -0x1.007a5f8f630e4p-3, 0x1.007a5f8f630e4p-3, 0x1.78a8d20a8b19dp-2, 0x1.2cb4f05c077f9p-1, 0x1.8a30aeed88f36p-1, 0x1.cee874ffb88b4p-1, 0x1.f68f1d8e42e81p-1, 0.0, 0.0, 0.0, 0.0},
    {-0x1.fa92c264d787ep-1, -0x1.e39f56616f9b0p-1, -0x1.bb3403514e483p-1, -0x1.82c45dda4726bp-1, -0x1.3c5a466d5e8b8p-1, -0x1.d50259a43a772p-2, -0x1.205cae642337cp-2, -0x1.852bd6676a9f9p-4, 0x1.852bd6676a9f9p-4, 0x1.205cae642337cp-2, 0x1.d50259a43a772p-2, 0x1.3c5a466d5e8b8p-1, 0x1.82c45dda4726bp-1, 0x1.bb3403514e483p-1, 0x1.e39f56616f9b0p-1, 0x1.fa92c264d787ep-1},
};
static const double GL_WEIGHTS[GL_NUM_ORDERS][16] = {
    {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.1c71c71c71c72p-1, 0x1.c71c71c71c71cp-1, 0x1.1c71c71c71c72p-1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.64340f7e7b66bp-2, 0x1.4de5f840c24cap-1, 0x1.4de5f840c24cap-1, 0x1.64340f7e7b66bp-2, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.e539ec36e038cp-3, 0x1.ea1da25ae415bp-2, 0x1.23456789abcdfp-1, 0x1.ea1da25ae415bp-2, 0x1.e539ec36e038cp-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.5edf601e2dbf8p-3, 0x1.716b7b5794c1cp-2, 0x1.df24d499545e8p-2, 0x1.df24d499545e8p-2, 0x1.716b7b5794c1cp-2, 0x1.5edf601e2dbf8p-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.9ea1d04ca0374p-4, 0x1.c76fb531d2b96p-3, 0x1.413c50a255615p-2, 0x1.736360b199343p-2, 0x1.736360b199343p-2, 0x1.413c50a255615p-2, 0x1.c76fb531d2b96p-3, 0x1.9ea1d04ca0374p-4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.1115f8b62dc1fp-4, 0x1.32138c878efe5p-3, 0x1.c0b059d00bc31p-3, 0x1.13baa7a559bfep-2, 0x1.2e9de7014d6efp-2, 0x1.2e9de7014d6efp-2, 0x1.13baa7a559bfep-2, 0x1.c0b059d00bc31p-3, 0x1.32138c878efe5p-3, 0x1.1115f8b62dc1fp-4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.8275d9dea6d8fp-5, 0x1.b60602bce6181p-4, 0x1.47d7258f22d8fp-3, 0x1.a0163e6b1ab72p-3, 0x1.de3155c256ab5p-3, 0x1.fe40ce6d4f025p-3, 0x1.fe40ce6d4f025p-3, 0x1.de3155c256ab5p-3, 0x1.a0163e6b1ab72p-3, 0x1.47d7258f22d8fp-3, 0x1.b60602bce6181p-4, 0x1.8275d9dea6d8fp-5, 0.0, 0.0, 0.0, 0.0},
    {0x1.bcddab4b7c211p-6, 0x1.fdfb1a2c1265dp-5, 0x1.85c4ee79cc258p-4, 0x1.fe7af2bad386ap-4, 0x1.325f61bca3cbfp-3, 0x1.5a6ebbb5a75fcp-3, 0x1.75f8c77e0c00fp-3, 0x1.83feae80e4dfcp-3, 0x1.83feae80e4dfcp-3, 0x1.75f8c77e0c00fp-3, 0x1.5a6ebbb5a75fcp-3, 0x1.325f61bca3cbfp-3, 0x1.fe7af2bad386ap-4, 0x1.85c4ee79cc258p-4, 0x1.fdfb1a2c1265dp-5, 0x1.bcddab4b7c211p-6},
};
#endif
