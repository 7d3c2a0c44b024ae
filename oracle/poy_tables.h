/* ORACLE / TEST INFRASTRUCTURE ONLY: restated POY cost tables (poy_tables.c). */
#ifndef POY_ORACLE_TABLES_H
#define POY_ORACLE_TABLES_H 1

/* Large enough for a 6-symbol bitset alphabet: 2 * (1 << 6) * (1 << 6). */
#define ORC_TABLE_SIZE 8192

typedef struct orc_tables {
    int alph;          /* symbols in the input matrix, gap last (5 for DNA) */
    int lcm;           /* bits per state; index = (a << lcm) + b */
    int gap;           /* gap bit (16 for DNA) */
    int a_sz;          /* number of states (31 for DNA) */
    int combinations;  /* 1: bitset states */
    int cost_model;    /* 0 linear, 1 affine */
    int gap_open;
    int is_metric, is_identity;
    int cost[ORC_TABLE_SIZE];
    int worst[ORC_TABLE_SIZE];
    int tail[ORC_TABLE_SIZE];
    int prepend[ORC_TABLE_SIZE];
    unsigned char median[ORC_TABLE_SIZE];
} orc_tables;

int orc_tables_build(orc_tables *t, const int *tcm, int alph, int gap_open);
int orc_tables_dna(orc_tables *t, int subs, int indel, int gap_open);
int orc_min_non0_cost(const orc_tables *t);

#endif
