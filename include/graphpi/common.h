// Small helpers of the reference's include/common.h.
#pragma once
#include <string>
#include "dataloader.h"
#include "pattern.h"

double get_wall_time();
void PatternType_printer(PatternType type);
bool is_equal_adj_mat(const int* adj_mat1, const int* adj_mat2, int size);
void GetDataType(DataType& type, const std::string str);
