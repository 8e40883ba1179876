// Source and receiver positions (ParallelFDTD src/base/SrcRec.h:33-168).
#ifndef PFDTD_SRCREC_H
#define PFDTD_SRCREC_H

#include <string>

#include "geomMath.h"

enum SrcType { SRC_HARD, SRC_SOFT, SRC_TRANSPARENT };
enum InputType { IMPULSE, GAUSSIAN, SINE, DATA };

class Position {
 public:
  Position() : p_(nv::Vec3f()) {}
  Position(float x, float y, float z) : p_(nv::Vec3f(x, y, z)) {}
  Position(float x, float y) : p_(nv::Vec3f(x, y, 0.f)) {}
  virtual ~Position() {}

  nv::Vec3f getP() { return p_; }

  // Element index on a grid with spacing dx = c / (fs * lambda), rounded
  // half up per axis (SrcRec.cpp:26-34).
  nv::Vec3i getElementIdx(unsigned spatial_fs, float c, float lambda);

 protected:
  nv::Vec3f p_;
};

class Source : public Position {
 public:
  Source() : Position(), source_type_(SRC_HARD), input_type_(IMPULSE), group_(0), input_data_idx_(0) {}
  Source(float x, float y, float z)
      : Position(x, y, z), source_type_(SRC_HARD), input_type_(IMPULSE), group_(0), input_data_idx_(0) {}
  Source(float x, float y, float z, enum SrcType source_type)
      : Position(x, y, z), source_type_(source_type), input_type_(IMPULSE), group_(0), input_data_idx_(0) {}
  Source(float x, float y, float z, enum SrcType source_type, unsigned int group)
      : Position(x, y, z), source_type_(source_type), input_type_(IMPULSE), group_(group), input_data_idx_(0) {}
  Source(float x, float y, float z, enum SrcType source_type, enum InputType input_type,
         unsigned int input_data_idx)
      : Position(x, y, z), source_type_(source_type), input_type_(input_type), group_(0),
        input_data_idx_(input_data_idx) {}
  Source(float x, float y)
      : Position(x, y), source_type_(SRC_HARD), input_type_(IMPULSE), group_(0), input_data_idx_(0) {}

  void setSourceType(enum SrcType source_type) { source_type_ = source_type; }
  void setInputType(enum InputType input_type) { input_type_ = input_type; }
  void setGroup(unsigned int group) { group_ = group; }
  void setInputDataIdx(unsigned int input_data_idx) { input_data_idx_ = input_data_idx; }
  unsigned int getInputDataIdx() const { return input_data_idx_; }
  enum SrcType getSourceType() const { return source_type_; }
  enum InputType getInputType() const { return input_type_; }
  unsigned int getGroup() const { return group_; }

 private:
  SrcType source_type_;
  InputType input_type_;
  unsigned int group_;
  unsigned int input_data_idx_;
};

class Receiver : public Position {
 public:
  Receiver() : Position() {}
  Receiver(float x, float y, float z) : Position(x, y, z) {}
  Receiver(float x, float y) : Position(x, y) {}
  void setOutputFp(std::string fp) { output_fp = fp; }

 private:
  std::string output_fp;
};

#endif
