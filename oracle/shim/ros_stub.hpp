// TEST INFRASTRUCTURE ONLY: minimal stand-ins for the ROS / tf2 types that the
// reference's headers and tsdf_evaluator.cpp name, so that the reference's own
// CPU sensor update and resampler compile without ROS.  None of these types
// carries arithmetic on the evaluated path except tf2::Quaternion::setRPY,
// which only feeds the mean-pose orientation (recorded in rpy_hook).
//
// <math.h> is deliberately not included: unqualified sin()/cos() on float in
// the reference then bind to the double-precision libm functions.
#ifndef TSDFL_ORACLE_ROS_STUB_HPP
#define TSDFL_ORACLE_ROS_STUB_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <unordered_set>
#include <stdexcept>
#include <string>
#include <vector>

namespace ros {
struct Duration {
    double d;
    explicit Duration(double v = 0) : d(v) {}
    double toSec() const { return d; }
};
struct Time {
    double t = 0;
    static Time now() { return Time(); }
    double toSec() const { return t; }
    bool operator==(const Time& o) const { return t == o.t; }
    Duration operator-(const Time& o) const { return Duration(t - o.t); }
};
inline std::ostream& operator<<(std::ostream& os, const Time& t) { return os << t.t; }
}  // namespace ros

#define ROS_ERROR_STREAM(x) (std::cerr << x << std::endl)
#define ROS_INFO_STREAM(x) (std::cerr << x << std::endl)
#define ROS_WARN_STREAM(x) (std::cerr << x << std::endl)
#define ROS_INFO(...) ((void)0)
#define ROS_WARN(...) ((void)0)
#define ROS_ERROR(...) ((void)0)

namespace std_msgs {
struct Header { ros::Time stamp; std::string frame_id; uint32_t seq = 0; };
}

namespace geometry_msgs {
struct Point { double x = 0, y = 0, z = 0; };
struct Vector3 { double x = 0, y = 0, z = 0; };
struct Quaternion { double x = 0, y = 0, z = 0, w = 1; };
struct Pose { Point position; Quaternion orientation; };
struct PoseWithCovariance { Pose pose; std::array<double, 36> covariance{}; };
struct Twist { Vector3 linear, angular; };
struct TwistWithCovariance { Twist twist; std::array<double, 36> covariance{}; };
struct Transform { Vector3 translation; Quaternion rotation; };
struct TransformStamped { std_msgs::Header header; std::string child_frame_id; Transform transform; };
}  // namespace geometry_msgs

namespace nav_msgs {
struct MapMetaData { float resolution = 0; uint32_t width = 0, height = 0; geometry_msgs::Pose origin; };
struct OccupancyGrid { std_msgs::Header header; MapMetaData info; std::vector<int8_t> data; };
struct Odometry { std_msgs::Header header; std::string child_frame_id; geometry_msgs::PoseWithCovariance pose; geometry_msgs::TwistWithCovariance twist; };
}  // namespace nav_msgs

namespace sensor_msgs {
struct PointField { std::string name; uint32_t offset = 0; uint8_t datatype = 0; uint32_t count = 0; };
struct PointCloud2 {
    std_msgs::Header header;
    uint32_t height = 0, width = 0;
    std::vector<PointField> fields;
    bool is_bigendian = false;
    uint32_t point_step = 0, row_step = 0;
    std::vector<uint8_t> data;
    bool is_dense = false;
};
struct Imu { std_msgs::Header header; geometry_msgs::Quaternion orientation; geometry_msgs::Vector3 angular_velocity, linear_acceleration; };

// Read-only field iterator over a PointCloud2 (only what tsdf_evaluator.cpp uses).
template <typename T>
class PointCloud2ConstIterator {
    const uint8_t* p_ = nullptr;
    const uint8_t* end_ = nullptr;
    uint32_t step_ = 1;
public:
    PointCloud2ConstIterator() = default;
    PointCloud2ConstIterator(const PointCloud2& c, const std::string& field) {
        uint32_t off = 0;
        for (const auto& f : c.fields) if (f.name == field) off = f.offset;
        step_ = c.point_step ? c.point_step : 1;
        p_ = c.data.data() + off;
        end_ = c.data.data() + off + (size_t)c.width * c.height * step_;
    }
    const T& operator[](size_t i) const { return reinterpret_cast<const T*>(p_)[i]; }
    PointCloud2ConstIterator& operator++() { p_ += step_; return *this; }
    bool operator!=(const PointCloud2ConstIterator& o) const { return p_ != o.p_; }
    PointCloud2ConstIterator end() const { PointCloud2ConstIterator e(*this); e.p_ = end_; return e; }
};
}  // namespace sensor_msgs

namespace tf2 {
// The last roll/pitch/yaw handed to setRPY, so tests can read the mean pose's
// orientation in the form the reference computed it.
inline double* rpy_hook() { static double v[3] = {0, 0, 0}; return v; }

struct TransformException : std::runtime_error {
    using std::runtime_error::runtime_error;
};

class Vector3 {
    double v_[3];
public:
    Vector3(double x = 0, double y = 0, double z = 0) : v_{x, y, z} {}
    double operator[](int i) const { return v_[i]; }
    double& operator[](int i) { return v_[i]; }
    double getX() const { return v_[0]; }
    double getY() const { return v_[1]; }
    double getZ() const { return v_[2]; }
};

class Quaternion {
public:
    double x = 0, y = 0, z = 0, w = 1;
    Quaternion() = default;
    Quaternion(double x_, double y_, double z_, double w_) : x(x_), y(y_), z(z_), w(w_) {}
    void setRPY(double roll, double pitch, double yaw) {
        rpy_hook()[0] = roll; rpy_hook()[1] = pitch; rpy_hook()[2] = yaw;
        double cr = std::cos(roll * 0.5), sr = std::sin(roll * 0.5);
        double cp = std::cos(pitch * 0.5), sp = std::sin(pitch * 0.5);
        double cy = std::cos(yaw * 0.5), sy = std::sin(yaw * 0.5);
        x = sr * cp * cy - cr * sp * sy;
        y = cr * sp * cy + sr * cp * sy;
        z = cr * cp * sy - sr * sp * cy;
        w = cr * cp * cy + sr * sp * sy;
    }
    double getX() const { return x; }
    double getY() const { return y; }
    double getZ() const { return z; }
    double getW() const { return w; }
};

class Matrix3x3 {
    Vector3 r_[3];
public:
    Matrix3x3() = default;
    explicit Matrix3x3(const Quaternion&) {}
    const Vector3& operator[](int i) const { return r_[i]; }
    Vector3& operator[](int i) { return r_[i]; }
    void getRPY(double& r, double& p, double& y) const { r = p = y = 0; }
};

class Transform {
    Matrix3x3 basis_;
    Vector3 origin_;
public:
    const Matrix3x3& getBasis() const { return basis_; }
    const Vector3& getOrigin() const { return origin_; }
    Transform inverse() const { return *this; }
};

// Inert: named by util.cpp's map-frame helpers, which no oracle path calls.
template <class A, class B>
inline void doTransform(const A&, B&, const geometry_msgs::TransformStamped&) {}
inline void convert(const Transform&, geometry_msgs::Transform&) {}

inline void convert(const Quaternion& a, geometry_msgs::Quaternion& b) { b.x = a.x; b.y = a.y; b.z = a.z; b.w = a.w; }
inline void convert(const geometry_msgs::Quaternion& a, Quaternion& b) { b = Quaternion(a.x, a.y, a.z, a.w); }
inline void convert(const geometry_msgs::Transform&, Transform&) {}
}  // namespace tf2

namespace tf2_ros {
struct Buffer {
    geometry_msgs::TransformStamped lookupTransform(const std::string&, const std::string&, const ros::Time&,
                                                    const ros::Duration&) const {
        throw tf2::TransformException("tf2 is not available in the oracle build");
    }
};
struct TransformListener { explicit TransformListener(Buffer&) {} };
struct TransformBroadcaster {};
}  // namespace tf2_ros

#endif
