/*
 * swm_index -- drop-in for SWMapper's serial_index (serial_index.c:811-865):
 *
 *     swm_index -i <reference.fa> -p <prefix> [-s<k>] [-h]
 *
 * builds the k-mer index on the GPU and writes the same seven files
 * (<prefix>.ref_info, .hash_count, .hash_offset, .positions, .pos_lseeds,
 * .base_2bits, .base_3bits). Exit status 0 on success, 1 on an error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "swmapper.h"

static void help(void) {
    printf("-i\tinput reference\n");
    printf("-p\tindex prefix\n");
    printf("-s\t[opt, default:12] seed length\n");
    exit(0);
}

int main(int argc, char *argv[]) {
    const char *ref = NULL, *prefix = NULL;
    unsigned k = 12;
    int opt;
    while ((opt = getopt(argc, argv, "h::i:s::p:")) != -1) {
        switch (opt) {
        case 'i': ref = optarg; break;
        case 'p': prefix = optarg; break;
        case 's':
            if (optarg) k = (unsigned)atoi(optarg);
            break;
        case 'h': help(); break;
        default: return 1;
        }
    }
    if (!ref || !prefix) {
        fprintf(stderr, "swm_index: -i <reference> and -p <prefix> are required\n");
        return 1;
    }
    const char *dev = getenv("SWM_DEVICE");
    int rc = swm_index_build_fasta(ref, prefix, k, dev ? atoi(dev) : 0);
    if (rc != SWM_OK) {
        fprintf(stderr, "swm_index: %s\n", swm_last_error());
        return 1;
    }
    return 0;
}
