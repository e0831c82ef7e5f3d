// hbt_average.e - event averaging of the HBT correlation files, with the
// command line of the reference's ebe_scripts/average_event_HBT_correlation_
// function.py: hbt_average.e working_folder results_folder.
#include <cstdio>

#include "hbt_host.h"

int main(int argc, char *argv[]) {
    if (argc < 3) {
        printf("Usage: %s working_folder results_folder\n", argv[0]);
        return 1;
    }
    const int n = hbt_host_average_events(argv[1], argv[2], 0);
    if (n < 0) return 1;
    printf("Analysis is done.\n");
    return 0;
}
