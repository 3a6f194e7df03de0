// The Boost.Thread names the reference sources use (boost::mutex and its
// scoped_lock), over a POSIX mutex (the reference sources are C++98).
// TEST INFRASTRUCTURE ONLY: lets the reference's ray-tracing sources
// compile where they lie for oracle/_ref.
#pragma once
#include <pthread.h>

namespace boost {
class mutex {
 public:
  mutex() { pthread_mutex_init(&m_, 0); }
  ~mutex() { pthread_mutex_destroy(&m_); }
  void lock() { pthread_mutex_lock(&m_); }
  void unlock() { pthread_mutex_unlock(&m_); }
  class scoped_lock {
   public:
    explicit scoped_lock(mutex& m) : m_(m) { m_.lock(); }
    ~scoped_lock() { m_.unlock(); }

   private:
    mutex& m_;
  };

 private:
  mutex(const mutex&);
  pthread_mutex_t m_;
};
}  // namespace boost
