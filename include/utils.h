/*
 * utils.h - drop-in for SMShovan/LabelPropCUDA headers/utils.h:41-78: the
 * command-line flags and the output files, with the reference's spelling,
 * defaults and text formats.
 */
#ifndef UTILS_H
#define UTILS_H

#include <string>

#include "graphTypes.h"

bool parseArguments(int argc, char *argv[], DynLPConfig &config);
void printConfig(const DynLPConfig &config);
bool ensureDirectory(const std::string &dirPath);
/* "<vertex> <label with 6 decimals>" per line */
bool writeLabelsToFile(const std::string &path, const float *labels, int numNodes);
/* header "batch,time_ms,accuracy", then "<b>,<ms 2 decimals>,<accuracy 6 decimals>" */
bool writeResultsCSV(const std::string &path, const float *batchTimes, const float *batchAccuracy,
                     int numBatches);

#endif /* UTILS_H */
