/* spx_rk_tables.h -- the Butcher tables a context may select (the reference's RK_INTEGRATOR_TYPE,
 * common/rk_config.hh:72-520), as exact hexadecimal doubles.
 *
 * The coefficients must equal the reference's to the last bit: identical inputs give identical
 * trajectories only with identical coefficients. tests/test_rk_tables.py compares every table with
 * the reference's own header compiled by oracle/ref_glue/rk_dump.cc. The layout is this library's:
 * per table its number, stages, order and adaptivity, then a[stages], the strictly lower triangle
 * of b row by row (the reference's RKSlopes reads b[i][j] for j < i only, src/trajectory_base.cc:
 * 315-357, so its implicit tables run as explicit ones with that triangle), v[stages] and
 * w[stages] (the lower-order weights of the adaptive tables, zero otherwise).
 *
 * Table 30 is absent: the reference's #if chain selects its Gauss-Legendre entry
 * (common/rk_config.hh:172), whose coefficients name an undeclared sqrtthr, so a reference build
 * with table 30 does not compile. Table 21's name string is one byte longer than its array, which
 * g++ accepts only with -fpermissive; its coefficients are valid and are taken from that build.
 * Plain C and C++: the oracle includes it too. */
#ifndef SPX_RK_TABLES_H
#define SPX_RK_TABLES_H

#define SPX_RK_MAX_STAGES 13
#define SPX_RK_N_TABLES 32

/* one table: number, stages, order, adaptive, offset of its coefficients in spx_rk_coeffs */
typedef struct { int number, stages, order, adaptive, offset; } spx_rk_entry;

#define SPX_RK_INDEX_INIT { \
   {0, 1, 1, 0, 0},  /* Euler */ \
   {1, 1, 1, 0, 3},  /* backward Euler */ \
   {2, 1, 2, 0, 6},  /* implicit midpoint */ \
   {3, 2, 2, 0, 9},  /* explicit midpoint */ \
   {4, 2, 2, 0, 16},  /* Kraaijevanger-Spijker */ \
   {5, 2, 2, 0, 23},  /* Qin-Zhang */ \
   {6, 2, 2, 0, 30},  /* Ralston 2 */ \
   {7, 2, 2, 0, 37},  /* Heun 2 */ \
   {8, 2, 2, 0, 44},  /* Crank-Nicolson */ \
   {9, 2, 2, 1, 51},  /* Heun-Euler 2(1) */ \
   {10, 2, 2, 1, 58},  /* Lobatto IIIA 2 */ \
   {11, 2, 2, 1, 65},  /* Lobatto IIIB 2 */ \
   {12, 2, 2, 1, 72},  /* Lobatto IIIC 2 */ \
   {13, 3, 2, 1, 79},  /* Fehlberg 2(1) */ \
   {14, 2, 3, 0, 91},  /* Radau IA 3 */ \
   {15, 2, 3, 0, 98},  /* Radau IIA 3 */ \
   {16, 3, 3, 0, 105},  /* Kutta 3 */ \
   {17, 3, 3, 0, 117},  /* Heun 3 */ \
   {18, 3, 3, 0, 129},  /* Ralston 3 */ \
   {19, 3, 3, 0, 141},  /* SSP 3 */ \
   {20, 4, 3, 0, 153},  /* implicit RK 3 */ \
   {21, 4, 3, 1, 171},  /* Bogacki-Shampine 3(2) */ \
   {22, 3, 4, 1, 189},  /* Lobatto IIIA 4 */ \
   {23, 3, 4, 1, 201},  /* Lobatto IIIB 4 */ \
   {24, 3, 4, 1, 213},  /* Lobatto IIIC 4 */ \
   {25, 4, 4, 0, 225},  /* classic RK4 */ \
   {26, 4, 4, 0, 243},  /* Kutta 3/8 */ \
   {27, 6, 5, 1, 261},  /* Runge-Kutta-Fehlberg 5(4) */ \
   {28, 6, 5, 1, 294},  /* Cash-Karp 5(4) */ \
   {29, 7, 5, 1, 327},  /* Dormand-Prince 5(4) */ \
   {31, 10, 7, 1, 369},  /* Runge-Kutta-Fehlberg 7(8) */ \
   {32, 13, 7, 1, 444},  /* Runge-Kutta-Fehlberg 8 (order 7 declared) */ \
}

/* per table: a[s], b[1][0], b[2][0..1], ..., b[s-1][0..s-2], v[s], w[s] */
#define SPX_RK_COEFFS_INIT { \
   /* 0: Euler */ \
   0.0, \
   0x1p+0, \
   0x1p+0, \
   /* 1: backward Euler */ \
   0x1p+0, \
   0x1p+0, \
   0x1p+0, \
   /* 2: implicit midpoint */ \
   0x1p-1, \
   0x1p+0, \
   0x1p+0, \
   /* 3: explicit midpoint */ \
   0.0, 0x1p-1, \
   0x1p-1, \
   0.0, 0x1p+0, \
   0.0, 0x1p+0, \
   /* 4: Kraaijevanger-Spijker */ \
   0x1p-1, 0x1.8p+0, \
   -0x1p-1, \
   -0x1p-1, 0x1.8p+0, \
   -0x1p-1, 0x1.8p+0, \
   /* 5: Qin-Zhang */ \
   0x1p-2, 0x1.8p-1, \
   0x1p-1, \
   0x1p-1, 0x1p-1, \
   0x1p-1, 0x1p-1, \
   /* 6: Ralston 2 */ \
   0.0, 0x1.5555555555555p-1, \
   0x1.5555555555555p-1, \
   0x1p-2, 0x1.8p-1, \
   0x1p-2, 0x1.8p-1, \
   /* 7: Heun 2 */ \
   0.0, 0x1p+0, \
   0x1p+0, \
   0x1p-1, 0x1p-1, \
   0x1p-1, 0x1p-1, \
   /* 8: Crank-Nicolson */ \
   0.0, 0x1p+0, \
   0x1p-1, \
   0x1p-1, 0x1p-1, \
   0x1p-1, 0x1p-1, \
   /* 9: Heun-Euler 2(1) */ \
   0.0, 0x1p+0, \
   0x1p+0, \
   0x1p+0, 0.0, \
   0x1p-1, 0x1p-1, \
   /* 10: Lobatto IIIA 2 */ \
   0.0, 0x1p+0, \
   0x1p-1, \
   0x1p+0, 0.0, \
   0x1p-1, 0x1p-1, \
   /* 11: Lobatto IIIB 2 */ \
   0x1p-1, 0x1p-1, \
   0x1p-1, \
   0x1p+0, 0.0, \
   0x1p-1, 0x1p-1, \
   /* 12: Lobatto IIIC 2 */ \
   0.0, 0x1p+0, \
   0x1p-1, \
   0x1p+0, 0.0, \
   0x1p-1, 0x1p-1, \
   /* 13: Fehlberg 2(1) */ \
   0.0, 0x1p-1, 0x1p+0, \
   0x1p-1, 0x1p-8, 0x1.fep-1, \
   0x1p-8, 0x1.fep-1, 0.0, \
   0x1p-9, 0x1.fep-1, 0x1p-9, \
   /* 14: Radau IA 3 */ \
   0.0, 0x1.5555555555555p-1, \
   0x1p-2, \
   0x1p-2, 0x1.8p-1, \
   0x1p-2, 0x1.8p-1, \
   /* 15: Radau IIA 3 */ \
   0x1.5555555555555p-2, 0x1p+0, \
   0x1.8p-1, \
   0x1.8p-1, 0x1p-2, \
   0x1.8p-1, 0x1p-2, \
   /* 16: Kutta 3 */ \
   0.0, 0x1p-1, 0x1p+0, \
   0x1p-1, -0x1p+0, 0x1p+1, \
   0x1.5555555555555p-3, 0x1.5555555555555p-1, 0x1.5555555555555p-3, \
   0x1.5555555555555p-3, 0x1.5555555555555p-1, 0x1.5555555555555p-3, \
   /* 17: Heun 3 */ \
   0.0, 0x1.5555555555555p-2, 0x1.5555555555555p-1, \
   0x1.5555555555555p-2, 0.0, 0x1.5555555555555p-1, \
   0x1p-2, 0.0, 0x1.8p-1, \
   0x1p-2, 0.0, 0x1.8p-1, \
   /* 18: Ralston 3 */ \
   0.0, 0x1p-1, 0x1.8p-1, \
   0x1p-1, 0.0, 0x1.8p-1, \
   0x1.c71c71c71c71cp-3, 0x1.5555555555555p-2, 0x1.c71c71c71c71cp-2, \
   0x1.c71c71c71c71cp-3, 0x1.5555555555555p-2, 0x1.c71c71c71c71cp-2, \
   /* 19: SSP 3 */ \
   0.0, 0x1p+0, 0x1p-1, \
   0x1p+0, 0x1p-2, 0x1p-2, \
   0x1.5555555555555p-3, 0x1.5555555555555p-3, 0x1.5555555555555p-1, \
   0x1.5555555555555p-3, 0x1.5555555555555p-3, 0x1.5555555555555p-1, \
   /* 20: implicit RK 3 */ \
   0x1p-1, 0x1.5555555555555p-1, 0x1p-1, 0x1p+0, \
   0x1.5555555555555p-3, -0x1p-1, 0x1p-1, 0x1.8p+0, \
   -0x1.8p+0, 0x1p-1, \
   0x1.8p+0, -0x1.8p+0, 0x1p-1, 0x1p-1, \
   0x1.8p+0, -0x1.8p+0, 0x1p-1, 0x1p-1, \
   /* 21: Bogacki-Shampine 3(2) */ \
   0.0, 0x1p-1, 0x1.8p-1, 0x1p+0, \
   0x1p-1, 0.0, 0x1.8p-1, 0x1.c71c71c71c71cp-3, \
   0x1.5555555555555p-2, 0x1.c71c71c71c71cp-2, \
   0x1.2aaaaaaaaaaabp-2, 0x1p-2, 0x1.5555555555555p-2, 0x1p-3, \
   0x1.c71c71c71c71cp-3, 0x1.5555555555555p-2, 0x1.c71c71c71c71cp-2, 0.0, \
   /* 22: Lobatto IIIA 4 */ \
   0.0, 0x1p-1, 0x1p+0, \
   0x1.aaaaaaaaaaaabp-3, 0x1.5555555555555p-3, 0x1.5555555555555p-1, \
   -0x1p-1, 0x1p+1, -0x1p-1, \
   0x1.5555555555555p-3, 0x1.5555555555555p-1, 0x1.5555555555555p-3, \
   /* 23: Lobatto IIIB 4 */ \
   0.0, 0x1p-1, 0x1p+0, \
   0x1.5555555555555p-3, 0x1.5555555555555p-3, 0x1.aaaaaaaaaaaabp-1, \
   -0x1p-1, 0x1p+1, -0x1p-1, \
   0x1.5555555555555p-3, 0x1.5555555555555p-1, 0x1.5555555555555p-3, \
   /* 24: Lobatto IIIC 4 */ \
   0.0, 0x1p-1, 0x1p+0, \
   0x1.5555555555555p-3, 0x1.5555555555555p-3, 0x1.5555555555555p-1, \
   -0x1p-1, 0x1p+1, -0x1p-1, \
   0x1.5555555555555p-3, 0x1.5555555555555p-1, 0x1.5555555555555p-3, \
   /* 25: classic RK4 */ \
   0.0, 0x1p-1, 0x1p-1, 0x1p+0, \
   0x1p-1, 0.0, 0x1p-1, 0.0, \
   0.0, 0x1p+0, \
   0x1.5555555555555p-3, 0x1.5555555555555p-2, 0x1.5555555555555p-2, 0x1.5555555555555p-3, \
   0x1.5555555555555p-3, 0x1.5555555555555p-2, 0x1.5555555555555p-2, 0x1.5555555555555p-3, \
   /* 26: Kutta 3/8 */ \
   0.0, 0x1.5555555555555p-2, 0x1.5555555555555p-1, 0x1p+0, \
   0x1.5555555555555p-2, -0x1.5555555555555p-2, 0x1p+0, 0x1p+0, \
   -0x1p+0, 0x1p+0, \
   0x1p-3, 0x1.8p-2, 0x1.8p-2, 0x1p-3, \
   0x1p-3, 0x1.8p-2, 0x1.8p-2, 0x1p-3, \
   /* 27: Runge-Kutta-Fehlberg 5(4) */ \
   0.0, 0x1p-2, 0x1.8p-2, 0x1.d89d89d89d89ep-1, \
   0x1p+0, 0x1p-1, \
   0x1p-2, 0x1.8p-4, 0x1.2p-2, 0x1.c23e39189614cp-1, \
   -0x1.a37b2a108bd3cp+1, 0x1.a912fe408db1p+1, 0x1.0425ed097b426p+1, -0x1p+3, \
   0x1.cb1a72c69cb1ap+2, -0x1.a5ad296b4a5adp-3, -0x1.2f684bda12f68p-2, 0x1p+1, \
   -0x1.61b58ba0961b6p+0, 0x1.cfd813f604fd8p-2, -0x1.199999999999ap-2, \
   0x1.e573ac901e574p-4, 0.0, 0x1.09b89459aa352p-1, 0x1.0323aaacfd498p-1, \
   -0x1.70a3d70a3d70ap-3, 0x1.29e4129e4129ep-5, \
   0x1.da12f684bda13p-4, 0.0, 0x1.190d13101190dp-1, 0x1.1216f485bd217p-1, \
   -0x1.999999999999ap-3, 0.0, \
   /* 28: Cash-Karp 5(4) */ \
   0.0, 0x1.999999999999ap-3, 0x1.3333333333333p-2, 0x1.3333333333333p-1, \
   0x1p+0, 0x1.cp-1, \
   0x1.999999999999ap-3, 0x1.3333333333333p-4, 0x1.ccccccccccccdp-3, 0x1.3333333333333p-2, \
   -0x1.ccccccccccccdp-1, 0x1.3333333333333p+0, -0x1.a12f684bda12fp-3, 0x1.4p+1, \
   -0x1.4bda12f684bdap+1, 0x1.4bda12f684bdap+0, 0x1.e3425ed097b42p-6, 0x1.5ep-2, \
   0x1.54bda12f684bep-5, 0x1.99f425ed097b4p-2, 0x1.fap-5, \
   0x1.90ee643b990eep-4, 0.0, 0x1.9c3d02e2bb28p-2, 0x1.aef9f76166929p-3, \
   0.0, 0x1.280a685dab4bp-2, \
   0x1.a284bda12f685p-4, 0.0, 0x1.891f2747c9d1fp-2, 0x1.f4ed097b425edp-3, \
   0x1.3c92492492492p-6, 0x1p-2, \
   /* 29: Dormand-Prince 5(4) */ \
   0.0, 0x1.999999999999ap-3, 0x1.3333333333333p-2, 0x1.999999999999ap-1, \
   0x1.c71c71c71c71cp-1, 0x1p+0, 0x1p+0, \
   0x1.999999999999ap-3, 0x1.3333333333333p-4, 0x1.ccccccccccccdp-3, 0x1.f49f49f49f49fp-1, \
   -0x1.ddddddddddddep+1, 0x1.c71c71c71c71cp+1, 0x1.79eec0fc37181p+1, -0x1.7310bd29520e4p+3, \
   0x1.3a552363c529p+3, -0x1.29c9eba1e3345p-2, 0x1.6c52bf5a814bp+1, -0x1.583e0f83e0f84p+3, \
   0x1.1d016a3721e8bp+3, 0x1.1d1745d1745d1p-2, -0x1.1818970d9cc2fp-2, 0x1.7555555555555p-4, \
   0.0, 0x1.cc0499a5605fbp-2, 0x1.4d55555555555p-1, -0x1.4a1cfb2b78c13p-2, \
   0x1.0c30c30c30c31p-3, \
   0x1.7555555555555p-4, 0.0, 0x1.cc0499a5605fbp-2, 0x1.4d55555555555p-1, \
   -0x1.4a1cfb2b78c13p-2, 0x1.0c30c30c30c31p-3, 0.0, \
   0x1.7048d159e26afp-4, 0.0, 0x1.d05f703aa30fap-2, 0x1.3a66666666666p-1, \
   -0x1.16075785e4908p-2, 0x1.6cbd323989ffp-4, 0x1.999999999999ap-6, \
   /* 31: Runge-Kutta-Fehlberg 7(8) */ \
   0.0, 0x1.f07c1f07c1f08p-5, 0x1.f07c1f07c1f08p-4, 0x1.745d1745d1746p-3, \
   0x1p-1, 0x1.5555555555555p-1, 0x1.b6db6db6db6dbp-1, 0x1p+0, \
   0.0, 0x1p+0, \
   0x1.f07c1f07c1f08p-5, 0.0, 0x1.f07c1f07c1f08p-4, 0x1.745d1745d1746p-5, \
   0.0, 0x1.1745d1745d174p-3, 0x1.58p-1, 0.0, \
   -0x1.4ap+1, 0x1.34p+1, -0x1.39cf8a021b641p+2, 0.0, \
   0x1.3c25ed097b426p+4, -0x1.eefe58315d28dp+3, 0x1.477cc3a64d5b6p+0, 0x1.0c9bab20f23efp+1, \
   0.0, -0x1.073af64c20d6fp+3, 0x1.bab4fbcfaf553p+2, -0x1.8726bbfd8082ap-2, \
   0x1.c117c6d9b8fd5p-2, -0x1.0a8ba2e8ba2e9p+2, 0.0, 0x1.1ap+4, \
   -0x1.cd36816816817p+3, 0x1.67109f959c428p+1, -0x1.a3ba2e8ba2e8cp+0, 0x1.92f70c880e526p-1, \
   0x1.5d1745d1745d1p-5, 0.0, 0.0, -0x1.deae6ae6ae6aep-4, \
   0x1.dec0d4c77b035p-3, -0x1.b9d1745d1745dp-3, 0x1.cc880e525982bp-5, 0.0, \
   -0x1.4d45d1745d174p+2, 0.0, 0x1.1ap+4, -0x1.c979249249249p+3, \
   0x1.4924924924925p+1, -0x1.6c8p+0, 0x1.762e8ba2e8ba3p-1, 0.0, \
   0x1p+0, \
   0x1.a12f684bda12fp-7, 0.0, 0.0, 0x1.2069113bbe669p-2, \
   0x1.3813813813814p-2, 0x1.84ccccccccccdp-4, 0x1.cbadbadbadbaep-3, 0.0, \
   0x1.4dbf86a314dcp-5, 0x1.4dbf86a314dcp-5, \
   0x1.b60b60b60b60bp-5, 0.0, 0.0, 0x1.2069113bbe669p-2, \
   0x1.3813813813814p-2, 0x1.84ccccccccccdp-4, 0x1.cbadbadbadbaep-3, 0x1.4dbf86a314dcp-5, \
   0.0, 0.0, \
   /* 32: Runge-Kutta-Fehlberg 8 (order 7 declared) */ \
   0.0, 0x1.2f684bda12f68p-4, 0x1.c71c71c71c71cp-4, 0x1.5555555555555p-3, \
   0x1.aaaaaaaaaaaabp-2, 0x1p-1, 0x1.aaaaaaaaaaaabp-1, 0x1.5555555555555p-3, \
   0x1.5555555555555p-1, 0x1.5555555555555p-2, 0x1p+0, 0.0, \
   0x1p+0, \
   0x1.2f684bda12f68p-4, 0x1.c71c71c71c71cp-6, 0x1.5555555555555p-4, 0x1.5555555555555p-5, \
   0.0, 0x1p-3, 0x1.aaaaaaaaaaaabp-2, 0.0, \
   -0x1.9p+0, 0x1.9p+0, 0x1.999999999999ap-5, 0.0, \
   0.0, 0x1p-2, 0x1.999999999999ap-3, -0x1.da12f684bda13p-3, \
   0.0, 0.0, 0x1.284bda12f684cp+0, -0x1.3425ed097b426p+1, \
   0x1.284bda12f684cp+1, 0x1.a740da740da74p-4, 0.0, 0.0, \
   0.0, 0x1.159e26af37c05p-2, -0x1.c71c71c71c71cp-3, 0x1.d950c83fb72eap-7, \
   0x1p+1, 0.0, 0.0, -0x1.1aaaaaaaaaaabp+3, \
   0x1.f49f49f49f49fp+3, -0x1.7c71c71c71c72p+3, 0x1.dc71c71c71c72p+2, 0x1.8p+1, \
   -0x1.af684bda12f68p-1, 0.0, 0.0, 0x1.b425ed097b426p-3, \
   -0x1.ceb240795ceb2p+2, 0x1.7097b425ed098p+2, -0x1.4444444444444p-2, 0x1.6aaaaaaaaaaabp+1, \
   -0x1.5555555555555p-4, 0x1.29959a9959a99p-1, 0.0, 0.0, \
   -0x1.0a2576a2576a2p+1, 0x1.18b9d18b9d18cp+2, -0x1.d5da895da895ep+1, 0x1.0a5d68a5d68a6p-1, \
   0x1.18f9c18f9c19p-1, 0x1.18f9c18f9c19p-2, 0x1.c18f9c18f9c19p-2, 0x1.df881df881df9p-7, \
   0.0, 0.0, 0.0, 0.0, \
   -0x1.2bb512bb512bbp-3, -0x1.df881df881df9p-7, -0x1.2bb512bb512bbp-4, 0x1.2bb512bb512bbp-4, \
   0x1.2bb512bb512bbp-3, 0.0, -0x1.bbd10bbd10bbdp-2, 0.0, \
   0.0, -0x1.0a2576a2576a2p+1, 0x1.a815fa815fa81p+1, -0x1.c31f3831f3832p+1, \
   0x1.11db891db891ep-1, 0x1.3e7063e7063e7p-1, 0x1.9c18f9c18f9c2p-3, 0x1.2bb512bb512bbp-2, \
   0.0, 0x1p+0, \
   0.0, 0.0, 0.0, 0.0, \
   0.0, 0x1.4b94b94b94b95p-2, 0x1.075075075075p-2, 0x1.075075075075p-2, \
   0x1.075075075075p-5, 0x1.075075075075p-5, 0.0, 0x1.8fd8fd8fd8fd9p-5, \
   0x1.8fd8fd8fd8fd9p-5, \
   0x1.8fd8fd8fd8fd9p-5, 0.0, 0.0, 0.0, \
   0.0, 0x1.4b94b94b94b95p-2, 0x1.075075075075p-2, 0x1.075075075075p-2, \
   0x1.075075075075p-5, 0x1.075075075075p-5, 0x1.8fd8fd8fd8fd9p-5, 0.0, \
   0.0, \
}

/* the tables as host arrays (device code places SPX_RK_COEFFS_INIT in constant memory) */
static const spx_rk_entry spx_rk_index[SPX_RK_N_TABLES] = SPX_RK_INDEX_INIT;
static const double spx_rk_coeffs[] = SPX_RK_COEFFS_INIT;

#endif
